// C ABI of the scan library (declared in include/gps.h).
//
// A plan plays the part of one constructed reference dispatcher
// (ChainedScanDecoupledLookbackDispatcher / ReduceThenScanDispatcher): it is
// created for a maximum size and owns the scratch memory the kernels need.
// Errors are returned as gps_status and described by gps_last_error(); the
// reference has no error reporting beyond printf
// (ChainedScanDecoupledLookbackDispatcher.cuh:117-120).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "gps_internal.h"

// Size classes of the autotuner: n within a factor of four share a class.
constexpr int kSizeClasses = 17;
inline int size_class(uint64_t n) {
    int bits = 0;
    while (n > 1 && bits < 64) {
        n >>= 1;
        ++bits;
    }
    return std::min(kSizeClasses - 1, bits / 2);
}

// Staging buffers of gps_scan_host, and their size in bytes (at most): six
// chunks of 32 MB keep copies in both directions and the scans going at once.
// Measured on GB300 with 1 GiB each way (pinned): either direction alone
// takes 5.09 / 5.56 ms, both at once 6.28 ms (the host link does not carry
// both at full rate). The scan of the array takes 6.76-6.89 ms with six
// 32 MB chunks, 6.73-6.93 with four of 64 MB, 7.01-7.04 with four of 16 MB,
// 7.5 with eight of 8 MB, 7.16 with two of 64 MB.
constexpr int kHostStages = 6;
constexpr uint64_t kHostChunkBytes = 32ull << 20;

struct gps_plan_s {
    gps_algo algo;
    gps_dtype dtype;
    uint64_t max_n;
    int device;
    int num_sms;
    uint32_t tile_elems;
    uint64_t capacity_tiles;
    void* scratch;        // WsHeader, then carry slots, then descriptors / tile sums
    size_t scratch_bytes;
    gps::WsHeader* hdr;
    void* carries;        // two elements (host-array scans)
    void* area;
    // Generic kernel (batched and floating-point scans): its workspace header
    // and 16-byte descriptors. On u32 chained-scan plans they are a region of
    // their own, with their own epoch, next to the 8-byte descriptors of the
    // u32 kernel; on other plans they are hdr and area.
    gps::WsHeader* hdr16;
    void* desc16;
    // Group descriptors of the generic kernel's fixed-order lookback, in the
    // same region after the unit descriptors (so that the epoch-wrap clear
    // covers them).
    void* group_desc16;
    // Integer chained-scan plans: the 16-byte, launch-tagged descriptors of
    // the one-tile-per-CTA kernels (mid.cu), one per tile; else null.
    void* desc_mid;
    void* group_desc_mid;  // and one per group of 32 tiles
    // Integer scans of at most this many elements run in one CTA (small.cu).
    uint64_t small_max;
    uint64_t mid_max;  // chained-scan plans: largest scan run as one tile per CTA
    // Autotuned launch configuration of the generic kernel per [segmented?]
    // [size class] (index into gps::kGenericCandidates; -1: not tuned).
    int8_t tuned[2][kSizeClasses];
    uint64_t wait_budget_ns;
    gps::StallConfig stall;
    gps::LaunchInfo last_launch;
    // Staging for gps_scan_host, created on first use.
    void* stage[kHostStages];
    uint64_t stage_elems;
    cudaStream_t copy_in, compute, copy_out;
    cudaEvent_t ev_loaded[kHostStages], ev_scanned[kHostStages], ev_free[kHostStages], ev_start, ev_done;
};

namespace {

thread_local std::string g_last_error;

gps_status fail(gps_status st, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return st;
}

gps_status cuda_fail(cudaError_t err, const char* what) {
    return fail(GPS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(err));
}

constexpr size_t kHeaderBytes = sizeof(gps::WsHeader);
constexpr size_t kCarryBytes = 128;  // two carry slots, padded to a line
constexpr uint64_t kDefaultBudgetNs = 1000000000ull;

size_t desc_bytes(gps_dtype dtype) { return dtype == GPS_DTYPE_U32 ? 8 : dtype == GPS_DTYPE_U32X4 ? 32 : 16; }

bool valid_dtype(int d) {
    return d == GPS_DTYPE_U32 || d == GPS_DTYPE_U64 || d == GPS_DTYPE_F32 || d == GPS_DTYPE_F32_COMPENSATED ||
           d == GPS_DTYPE_U32X4;
}
bool is_float(gps_dtype d) { return d == GPS_DTYPE_F32 || d == GPS_DTYPE_F32_COMPENSATED; }
// Types whose every scan runs on the generic kernel (no L2, one-CTA or
// reduce-then-scan kernel of their own).
bool generic_only(gps_dtype d) { return is_float(d) || d == GPS_DTYPE_U32X4; }

// Launch configuration of the generic kernel for a scan of n elements: the
// autotuned one of the size class if there is one, else the default rule.
gps::GenericConfig generic_config(const gps_plan_s* p, bool segmented, uint64_t n) {
    const int c = p->tuned[segmented ? 1 : 0][size_class(n)];
    if (c >= 0 && c < gps::kNumGenericCandidates) return gps::kGenericCandidates[c];
    return gps::default_generic_config(n, p->tile_elems, p->num_sms);
}

// Generic kernel (scan_seg.cuh): floating-point scans and batched scans.
cudaError_t launch_generic(gps_dtype dtype, bool inclusive, const gps::ScanArgs& a, const gps::SegArgs* sg,
                           const gps::GenericConfig& cfg, int num_sms, cudaStream_t stream, gps::LaunchInfo* info) {
    switch (dtype) {
        case GPS_DTYPE_U32: return gps::launch_seg_u32(inclusive, a, sg, cfg, num_sms, stream, info);
        case GPS_DTYPE_U64: return gps::launch_seg_u64(inclusive, a, sg, cfg, num_sms, stream, info);
        case GPS_DTYPE_F32: return gps::launch_seg_f32(inclusive, a, sg, cfg, num_sms, stream, info);
        case GPS_DTYPE_F32_COMPENSATED: return gps::launch_seg_f32c(inclusive, a, sg, cfg, num_sms, stream, info);
        case GPS_DTYPE_U32X4: return gps::launch_seg_u32x4(inclusive, a, sg, cfg, num_sms, stream, info);
    }
    return cudaErrorInvalidValue;
}
// Whether a launch configuration's kernels exist for the element type (two
// threads per row do not fit every type's shared memory).
bool generic_config_fits(gps_dtype dtype, const gps::GenericConfig& cfg) {
    if (cfg.split == 1) return true;
    switch (dtype) {
        case GPS_DTYPE_U32: return gps::seg_u32_x2_fits(cfg.unit);
        case GPS_DTYPE_U64: return gps::seg_u64_x2_fits(cfg.unit);
        case GPS_DTYPE_F32: return gps::seg_f32_x2_fits(cfg.unit);
        case GPS_DTYPE_F32_COMPENSATED: return gps::seg_f32c_x2_fits(cfg.unit);
        case GPS_DTYPE_U32X4: return gps::seg_u32x4_x2_fits(cfg.unit);
    }
    return false;
}
bool valid_algo(int a) { return a == GPS_ALGO_CSDL || a == GPS_ALGO_RTS; }
bool valid_kind(int k) { return k == GPS_SCAN_EXCLUSIVE || k == GPS_SCAN_INCLUSIVE; }

gps_status check_device(const gps_plan_s* p) {
    int dev = -1;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return cuda_fail(err, "cudaGetDevice");
    if (dev != p->device)
        return fail(GPS_ERR_WRONG_DEVICE, "plan was created on device %d but device %d is current", p->device, dev);
    return GPS_OK;
}

// Device-side launch of one scan of n elements (n >= 1, already validated).
gps_status launch_scan(gps_plan_s* p, bool inclusive, const void* in, void* out, uint64_t n, const void* carry_in,
                       void* carry_out, cudaStream_t stream) {
    gps::ScanArgs a{};
    a.in = in;
    a.out = out;
    a.n = n;
    a.num_tiles = static_cast<uint32_t>((n + p->tile_elems - 1) / p->tile_elems);
    a.hdr = p->hdr;
    a.desc = p->area;
    a.spine = nullptr;
    a.carry_in = carry_in;
    a.carry_out = carry_out;
    a.wait_budget_ns = p->wait_budget_ns;
    a.stall = p->stall;
    cudaError_t err;
    if (generic_only(p->dtype)) {
        a.hdr = p->hdr16;
        a.desc = p->desc16;
        a.group_desc = p->group_desc16;
        err = launch_generic(p->dtype, inclusive, a, nullptr, generic_config(p, false, n), p->num_sms, stream,
                             &p->last_launch);
    } else if (n <= p->small_max && p->stall.mode == 0 && p->stall.fallback_polls == 0) {
        err = gps::launch_small(p->dtype, inclusive, a, stream, &p->last_launch);
    } else if (p->algo == GPS_ALGO_CSDL && n <= p->mid_max && p->stall.mode == 0 && p->stall.fallback_polls == 0) {
        a.desc = p->desc_mid;
        a.group_desc = p->group_desc_mid;
        err = gps::launch_mid(p->dtype, inclusive, a, p->num_sms, stream, &p->last_launch);
    } else if (p->algo == GPS_ALGO_CSDL) {
        err = gps::launch_csdl(p->dtype, inclusive, p->stall.mode != 0 || p->stall.fallback_polls != 0, a, p->num_sms,
                               stream, &p->last_launch);
    } else {
        err = gps::launch_rts(p->dtype, inclusive, a, p->area, p->num_sms, stream, &p->last_launch);
    }
    if (err != cudaSuccess) return cuda_fail(err, "scan launch");
    return GPS_OK;
}

// Order-free 64-bit hash of a buffer (the sum of x_i * (2i + 1) over its
// 8-byte words, mod 2^64), added into *h: the autotuner compares each launch
// configuration's output with the first one's without keeping a copy.
__global__ void hash_words_kernel(const uint64_t* w, uint64_t nwords, const uint8_t* tail, uint32_t tail_bytes,
                                  unsigned long long* h) {
    uint64_t acc = 0;
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < nwords;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        acc += w[i] * (2 * i + 1);
    if (blockIdx.x == 0 && threadIdx.x == 0)
        for (uint32_t b = 0; b < tail_bytes; ++b) acc += static_cast<uint64_t>(tail[b]) * (2 * (nwords + b) + 1);
#pragma unroll
    for (int m = 16; m; m >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, m);
    if ((threadIdx.x & 31u) == 0) atomicAdd(h, static_cast<unsigned long long>(acc));
}

// Hash of `bytes` bytes at d (8-byte aligned) into *d_hash, on `stream`.
cudaError_t hash_buffer(const void* d, uint64_t bytes, unsigned long long* d_hash, cudaStream_t stream) {
    cudaError_t err = cudaMemsetAsync(d_hash, 0, sizeof(*d_hash), stream);
    if (err != cudaSuccess) return err;
    const uint64_t nwords = bytes / 8;
    hash_words_kernel<<<304, 256, 0, stream>>>(static_cast<const uint64_t*>(d), nwords,
                                                static_cast<const uint8_t*>(d) + nwords * 8,
                                                static_cast<uint32_t>(bytes % 8), d_hash);
    return cudaGetLastError();
}

}  // namespace

namespace gps {
size_t dtype_size(gps_dtype dtype) { return dtype == GPS_DTYPE_U64 ? 8 : dtype == GPS_DTYPE_U32X4 ? 16 : 4; }
GenericConfig default_generic_config(uint64_t n, uint32_t tile_elems, int num_sms) {
    const uint64_t units4 = (n + 4ull * tile_elems - 1) / (4ull * tile_elems);
    return units4 >= 2ull * static_cast<uint64_t>(num_sms) ? GenericConfig{4, 1, 1} : GenericConfig{1, 1, 1};
}
void record_error(const char* msg) { g_last_error = msg; }
}  // namespace gps

extern "C" {

int gps_version(void) { return 10000; }

const char* gps_status_string(gps_status status) {
    switch (status) {
        case GPS_OK: return "GPS_OK";
        case GPS_ERR_INVALID_ARGUMENT: return "GPS_ERR_INVALID_ARGUMENT";
        case GPS_ERR_SIZE_EXCEEDS_PLAN: return "GPS_ERR_SIZE_EXCEEDS_PLAN";
        case GPS_ERR_CUDA: return "GPS_ERR_CUDA";
        case GPS_ERR_TIMEOUT: return "GPS_ERR_TIMEOUT";
        case GPS_ERR_UNSUPPORTED: return "GPS_ERR_UNSUPPORTED";
        case GPS_ERR_OUT_OF_MEMORY: return "GPS_ERR_OUT_OF_MEMORY";
        case GPS_ERR_WRONG_DEVICE: return "GPS_ERR_WRONG_DEVICE";
    }
    return "GPS_ERR_UNKNOWN";
}

const char* gps_last_error(void) { return g_last_error.c_str(); }

gps_status gps_plan_create(gps_plan* out_plan, gps_algo algo, gps_dtype dtype, uint64_t max_n) {
    if (out_plan == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "out_plan is NULL");
    *out_plan = nullptr;
    if (!valid_algo(algo)) return fail(GPS_ERR_INVALID_ARGUMENT, "unknown algorithm %d", static_cast<int>(algo));
    if (!valid_dtype(dtype)) return fail(GPS_ERR_INVALID_ARGUMENT, "unknown dtype %d", static_cast<int>(dtype));
    if (max_n == 0) return fail(GPS_ERR_INVALID_ARGUMENT, "max_n must be at least 1");
    if (generic_only(dtype) && algo != GPS_ALGO_CSDL)
        return fail(GPS_ERR_UNSUPPORTED, "floating-point and struct scans use the chained scan (GPS_ALGO_CSDL)");
    const uint32_t tile = algo == GPS_ALGO_CSDL ? gps::csdl_tile_elems(dtype) : gps::rts_tile_elems(dtype);
    const uint64_t tiles = (max_n + tile - 1) / tile;
    if (tiles >= (1ull << 31))
        return fail(GPS_ERR_INVALID_ARGUMENT, "max_n %llu needs %llu tiles; the limit is 2^31 - 1",
                    static_cast<unsigned long long>(max_n), static_cast<unsigned long long>(tiles));

    gps_plan_s* p = new (std::nothrow) gps_plan_s();
    if (p == nullptr) return fail(GPS_ERR_OUT_OF_MEMORY, "host allocation failed");
    p->algo = algo;
    p->dtype = dtype;
    p->max_n = max_n;
    p->tile_elems = tile;
    p->capacity_tiles = tiles;
    p->wait_budget_ns = kDefaultBudgetNs;
    std::memset(p->tuned, -1, sizeof(p->tuned));
    // Chained-scan plans send small integer scans to the one-tile-per-CTA
    // kernel too: measured on GB300 it matches or beats the one-CTA kernel
    // at every size up to 64 KB (2.0 against 2.2-2.35 us up to one tile,
    // 2.7 against 4.5 us at 16384 u32). Reduce-then-scan plans keep the
    // one-CTA kernel for small inputs.
    p->small_max = algo == GPS_ALGO_CSDL ? 0 : gps::small_scan_max_elems(dtype);
    p->mid_max = algo == GPS_ALGO_CSDL && !generic_only(dtype) ? gps::kMidMaxBytes / gps::dtype_size(dtype) : 0;
    cudaError_t err = cudaGetDevice(&p->device);
    if (err == cudaSuccess) err = cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount, p->device);
    if (err != cudaSuccess) {
        delete p;
        return cuda_fail(err, "device query");
    }
    // Chained scan: one descriptor per tile plus the lookback padding;
    // reduce-then-scan: one tile sum per tile.
    // Generic-kernel descriptors (packed, or one per line for launches of few
    // units) are followed by the group descriptors of its lookback; both are
    // counted in 16-byte words.
    const size_t per_tile = algo == GPS_ALGO_CSDL ? desc_bytes(dtype) : gps::dtype_size(dtype);
    const uint64_t seg_dw = (dtype == GPS_DTYPE_U32 ? 16 : per_tile) / 16;  // words per generic descriptor
    const uint64_t seg_units = gps::seg_desc_words(tiles, seg_dw), seg_groups = gps::seg_group_words(tiles, seg_dw);
    const uint64_t slots = algo == GPS_ALGO_CSDL ? (dtype != GPS_DTYPE_U32 ? (seg_units + seg_groups) / seg_dw
                                                                          : tiles + gps::kDescPad)
                                                 : tiles;
    // u32 chained-scan plans keep 8-byte descriptors; batched scans of them
    // use the generic kernel's 16-byte descriptors, kept in a region of their
    // own so that the two formats never meet in one slot.
    const uint64_t slots16 = (algo == GPS_ALGO_CSDL && dtype == GPS_DTYPE_U32) ? seg_units + seg_groups : 0;
    // One-tile-per-CTA kernels of integer chained-scan plans: 16-byte
    // descriptors tagged with the launch, in a region no other kernel uses.
    const uint64_t slots_mid = (algo == GPS_ALGO_CSDL && !generic_only(dtype)) ? tiles + gps::kDescPad : 0;
    const uint64_t groups_mid = slots_mid ? (tiles + 31) / 32 + gps::kDescPad : 0;
    // [header][carries][descriptors or tile sums]; for u32 chained-scan
    // plans, [256-byte aligned: generic header][16-byte descriptors]; for
    // integer chained-scan plans, [256-byte aligned: mid-size descriptors].
    const size_t main_bytes = kHeaderBytes + kCarryBytes + slots * per_tile;
    const size_t region16 = (main_bytes + 255) & ~static_cast<size_t>(255);
    const size_t end16 = slots16 ? region16 + kHeaderBytes + slots16 * 16 : main_bytes;
    const size_t region_mid = (end16 + 255) & ~static_cast<size_t>(255);
    const uint64_t words_mid = slots_mid ? gps::mid_desc_words(tiles) : 0;
    p->scratch_bytes = slots_mid ? region_mid + (words_mid + groups_mid * gps::kMidDescStride) * 16 : end16;
    err = cudaMalloc(&p->scratch, p->scratch_bytes);
    if (err != cudaSuccess) {
        const size_t bytes = p->scratch_bytes;
        delete p;
        return fail(err == cudaErrorMemoryAllocation ? GPS_ERR_OUT_OF_MEMORY : GPS_ERR_CUDA, "cudaMalloc(%zu): %s",
                    bytes, cudaGetErrorString(err));
    }
    p->hdr = static_cast<gps::WsHeader*>(p->scratch);
    p->carries = static_cast<char*>(p->scratch) + kHeaderBytes;
    p->area = static_cast<char*>(p->scratch) + kHeaderBytes + kCarryBytes;
    p->hdr16 = slots16 ? reinterpret_cast<gps::WsHeader*>(static_cast<char*>(p->scratch) + region16) : p->hdr;
    p->desc16 = slots16 ? static_cast<char*>(p->scratch) + region16 + kHeaderBytes : p->area;
    if (algo == GPS_ALGO_CSDL) p->group_desc16 = static_cast<char*>(p->desc16) + seg_units * 16;
    p->desc_mid = slots_mid ? static_cast<char*>(p->scratch) + region_mid : nullptr;
    p->group_desc_mid = slots_mid ? static_cast<char*>(p->scratch) + region_mid + words_mid * 16 : nullptr;
    gps::WsHeader h{};
    h.epoch = 1;
    h.capacity_tiles = slots;
    err = cudaMemset(p->scratch, 0, p->scratch_bytes);
    if (err == cudaSuccess) err = cudaMemcpy(p->hdr, &h, sizeof(h), cudaMemcpyHostToDevice);
    if (err == cudaSuccess && slots16) {
        h.capacity_tiles = slots16;
        err = cudaMemcpy(p->hdr16, &h, sizeof(h), cudaMemcpyHostToDevice);
    }
    if (err == cudaSuccess) err = cudaDeviceSynchronize();
    if (err != cudaSuccess) {
        cudaFree(p->scratch);
        delete p;
        return cuda_fail(err, "scratch initialisation");
    }
    *out_plan = p;
    return GPS_OK;
}

gps_status gps_plan_destroy(gps_plan p) {
    if (p == nullptr) return GPS_OK;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(p->device);
    cudaError_t err = cudaFree(p->scratch);
    for (int b = 0; b < kHostStages; ++b) {
        if (p->stage[b]) cudaFree(p->stage[b]);
        if (p->ev_loaded[b]) cudaEventDestroy(p->ev_loaded[b]);
        if (p->ev_scanned[b]) cudaEventDestroy(p->ev_scanned[b]);
        if (p->ev_free[b]) cudaEventDestroy(p->ev_free[b]);
    }
    if (p->ev_start) cudaEventDestroy(p->ev_start);
    if (p->ev_done) cudaEventDestroy(p->ev_done);
    if (p->copy_in) cudaStreamDestroy(p->copy_in);
    if (p->compute) cudaStreamDestroy(p->compute);
    if (p->copy_out) cudaStreamDestroy(p->copy_out);
    if (prev >= 0) cudaSetDevice(prev);
    delete p;
    if (err != cudaSuccess) return cuda_fail(err, "cudaFree");
    return GPS_OK;
}

gps_status gps_plan_scratch_bytes(gps_plan p, size_t* out_bytes) {
    if (p == nullptr || out_bytes == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "NULL argument");
    *out_bytes = p->scratch_bytes;
    return GPS_OK;
}

gps_status gps_scan(gps_plan p, gps_scan_kind kind, const void* d_in, void* d_out, uint64_t n, gps_stream_t stream) {
    if (p == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (!valid_kind(kind)) return fail(GPS_ERR_INVALID_ARGUMENT, "unknown scan kind %d", static_cast<int>(kind));
    if (n == 0) return GPS_OK;
    if (n > p->max_n)
        return fail(GPS_ERR_SIZE_EXCEEDS_PLAN, "requested size %llu exceeds the plan's maximum %llu",
                    static_cast<unsigned long long>(n), static_cast<unsigned long long>(p->max_n));
    if (d_in == nullptr || d_out == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "NULL data pointer");
    const size_t es = gps::dtype_size(p->dtype);
    const uintptr_t i = reinterpret_cast<uintptr_t>(d_in), o = reinterpret_cast<uintptr_t>(d_out);
    if ((i % es) != 0 || (o % es) != 0)
        return fail(GPS_ERR_INVALID_ARGUMENT, "pointers must be aligned to the %zu-byte element size", es);
    const uint64_t bytes = n * es;
    if (i != o && i < o + bytes && o < i + bytes)
        return fail(GPS_ERR_INVALID_ARGUMENT, "input and output overlap without being identical");
    if (generic_only(p->dtype) && ((i | o) & 15u) != 0)
        return fail(GPS_ERR_INVALID_ARGUMENT, "floating-point and struct scans need 16-byte aligned buffers");
    gps_status st = check_device(p);
    if (st != GPS_OK) return st;
    return launch_scan(p, kind == GPS_SCAN_INCLUSIVE, d_in, d_out, n, nullptr, nullptr,
                       reinterpret_cast<cudaStream_t>(stream));
}

namespace {

// Validates a batched (d_offsets != NULL) or generic-kernel plain scan and
// fills its kernel arguments. Returns GPS_OK with n == 0 meaning "nothing to do".
gps_status prepare_generic(gps_plan_s* p, gps_scan_kind kind, const void* d_in, void* d_out, uint64_t n,
                           const uint32_t* d_offsets, uint64_t num_segments, gps::ScanArgs* a, gps::SegArgs* sg) {
    if (p == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (!valid_kind(kind)) return fail(GPS_ERR_INVALID_ARGUMENT, "unknown scan kind %d", static_cast<int>(kind));
    if (p->algo != GPS_ALGO_CSDL)
        return fail(GPS_ERR_UNSUPPORTED, "batched scans run on chained-scan plans (GPS_ALGO_CSDL)");
    if (d_offsets == nullptr && !generic_only(p->dtype))
        return fail(GPS_ERR_UNSUPPORTED, "integer plans use the generic kernel for batched scans only");
    if (n == 0) return GPS_OK;
    if (d_offsets != nullptr && num_segments == 0)
        return fail(GPS_ERR_INVALID_ARGUMENT, "%llu elements but no segments", static_cast<unsigned long long>(n));
    if (n > p->max_n)
        return fail(GPS_ERR_SIZE_EXCEEDS_PLAN, "requested size %llu exceeds the plan's maximum %llu",
                    static_cast<unsigned long long>(n), static_cast<unsigned long long>(p->max_n));
    if (d_offsets != nullptr && (n > 0xFFFFFFFFull || num_segments > 0xFFFFFFFEull))
        return fail(GPS_ERR_INVALID_ARGUMENT, "uint32 offsets limit a batch to 2^32 - 1 elements");
    if (d_in == nullptr || d_out == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "NULL pointer");
    const size_t es = gps::dtype_size(p->dtype);
    const uintptr_t i = reinterpret_cast<uintptr_t>(d_in), o = reinterpret_cast<uintptr_t>(d_out);
    if (((i | o) & 15u) != 0) return fail(GPS_ERR_INVALID_ARGUMENT, "this scan needs 16-byte aligned buffers");
    if ((reinterpret_cast<uintptr_t>(d_offsets) & 3u) != 0)
        return fail(GPS_ERR_INVALID_ARGUMENT, "offsets must be 4-byte aligned");
    const uint64_t bytes = n * es;
    if (i != o && i < o + bytes && o < i + bytes)
        return fail(GPS_ERR_INVALID_ARGUMENT, "input and output overlap without being identical");
    gps_status st = check_device(p);
    if (st != GPS_OK) return st;
    if (((reinterpret_cast<uintptr_t>(p->desc16) | reinterpret_cast<uintptr_t>(p->group_desc16)) & 15u) != 0)
        return fail(GPS_ERR_CUDA, "internal: misaligned descriptor region");
    *a = gps::ScanArgs{};
    a->in = d_in;
    a->out = d_out;
    a->n = n;
    a->num_tiles = static_cast<uint32_t>((n + p->tile_elems - 1) / p->tile_elems);
    a->hdr = p->hdr16;
    a->desc = p->desc16;
    a->group_desc = p->group_desc16;
    a->wait_budget_ns = p->wait_budget_ns;
    *sg = gps::SegArgs{d_offsets, static_cast<uint32_t>(num_segments)};
    return GPS_OK;
}

}  // namespace

gps_status gps_scan_segmented(gps_plan p, gps_scan_kind kind, const void* d_in, void* d_out, uint64_t n,
                              const uint32_t* d_offsets, uint64_t num_segments, gps_stream_t stream) {
    if (d_offsets == nullptr && n != 0) return fail(GPS_ERR_INVALID_ARGUMENT, "NULL offsets");
    gps::ScanArgs a;
    gps::SegArgs sg;
    gps_status st = prepare_generic(p, kind, d_in, d_out, n, d_offsets, num_segments, &a, &sg);
    if (st != GPS_OK || n == 0) return st;
    const cudaError_t err = launch_generic(p->dtype, kind == GPS_SCAN_INCLUSIVE, a, &sg, generic_config(p, true, n),
                                           p->num_sms, reinterpret_cast<cudaStream_t>(stream), &p->last_launch);
    if (err != cudaSuccess) return cuda_fail(err, "batched scan launch");
    return GPS_OK;
}

gps_status gps_plan_autotune(gps_plan p, gps_scan_kind kind, const void* d_in, void* d_out, uint64_t n,
                             const uint32_t* d_offsets, uint64_t num_segments, gps_stream_t stream,
                             uint32_t* out_unit, uint32_t* out_ctas, uint32_t* out_threads_per_row) {
    gps::ScanArgs a;
    gps::SegArgs sg;
    gps_status st = prepare_generic(p, kind, d_in, d_out, n, d_offsets, num_segments, &a, &sg);
    if (st != GPS_OK) return st;
    if (n == 0) return fail(GPS_ERR_INVALID_ARGUMENT, "nothing to tune for n == 0");
    const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaError_t err = cudaStreamIsCapturing(s, &cap);
    if (err != cudaSuccess) return cuda_fail(err, "cudaStreamIsCapturing");
    if (cap != cudaStreamCaptureStatusNone) return fail(GPS_ERR_INVALID_ARGUMENT, "autotuning cannot be captured");
    if (d_in == d_out) return fail(GPS_ERR_INVALID_ARGUMENT, "autotuning needs separate input and output buffers");
    const bool seg = d_offsets != nullptr;
    // Integer results do not depend on the launch configuration: every
    // candidate's output must hash like the first one's, or the candidate is
    // not taken. (Floating-point results differ in rounding from one
    // configuration to the next.)
    const bool check = !is_float(p->dtype);
    unsigned long long* d_hash = reinterpret_cast<unsigned long long*>(p->carries);
    const uint64_t out_bytes = n * gps::dtype_size(p->dtype);
    unsigned long long first_hash = 0, hash = 0;
    bool have_first = false;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    err = cudaEventCreate(&e0);
    if (err == cudaSuccess) err = cudaEventCreate(&e1);
    int best = -1, rejected = 0;
    float best_ms = 0.0f;
    for (int c = 0; c < gps::kNumGenericCandidates && err == cudaSuccess; ++c) {
        const gps::GenericConfig& cfg = gps::kGenericCandidates[c];
        if (!generic_config_fits(p->dtype, cfg)) continue;  // this kernel shape does not fit the type
        gps::LaunchInfo info{};
        const gps::SegArgs* sgp = seg ? &sg : nullptr;
        const bool incl = kind == GPS_SCAN_INCLUSIVE;
        err = launch_generic(p->dtype, incl, a, sgp, cfg, p->num_sms, s, &info);  // warm-up
        if (err == cudaSuccess && check) {
            err = hash_buffer(d_out, out_bytes, d_hash, s);
            if (err == cudaSuccess) err = cudaMemcpyAsync(&hash, d_hash, sizeof(hash), cudaMemcpyDeviceToHost, s);
            if (err == cudaSuccess) err = cudaStreamSynchronize(s);
            if (err == cudaSuccess && !have_first) {
                first_hash = hash;
                have_first = true;
            }
        }
        if (err == cudaSuccess) err = cudaEventRecord(e0, s);
        for (int r = 0; r < 3 && err == cudaSuccess; ++r)
            err = launch_generic(p->dtype, incl, a, sgp, cfg, p->num_sms, s, &info);
        if (err == cudaSuccess) err = cudaEventRecord(e1, s);
        if (err == cudaSuccess) err = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
        if (err != cudaSuccess) break;
        if (check && hash != first_hash) {
            ++rejected;
            continue;
        }
        if (best < 0 || ms < best_ms) {
            best = c;
            best_ms = ms;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (err != cudaSuccess) return cuda_fail(err, "autotuning");
    if (best < 0) return fail(GPS_ERR_CUDA, "autotuning: no launch configuration ran");
    // Leave a correct result in d_out, from the chosen configuration.
    err = launch_generic(p->dtype, kind == GPS_SCAN_INCLUSIVE, a, seg ? &sg : nullptr, gps::kGenericCandidates[best],
                         p->num_sms, s, &p->last_launch);
    if (err != cudaSuccess) return cuda_fail(err, "autotuning");
    p->tuned[seg ? 1 : 0][size_class(n)] = static_cast<int8_t>(best);
    if (out_unit) *out_unit = gps::kGenericCandidates[best].unit;
    if (out_ctas) *out_ctas = gps::kGenericCandidates[best].ctas_div;
    if (out_threads_per_row) *out_threads_per_row = gps::kGenericCandidates[best].split;
    st = gps_plan_check(p, stream);
    if (st != GPS_OK) return st;
    if (rejected != 0)
        return fail(GPS_ERR_CUDA, "autotuning: %d launch configuration(s) gave a different result and were not taken",
                    rejected);
    return GPS_OK;
}

gps_status gps_plan_set_generic_config(gps_plan p, int segmented, uint64_t n, uint32_t unit, uint32_t ctas_div,
                                       uint32_t threads_per_row) {
    if (p == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "plan is NULL");
    for (int c = 0; c < gps::kNumGenericCandidates; ++c) {
        const gps::GenericConfig& g = gps::kGenericCandidates[c];
        if (g.unit == unit && g.ctas_div == ctas_div && g.split == threads_per_row) {
            if (!generic_config_fits(p->dtype, g))
                return fail(GPS_ERR_UNSUPPORTED, "%u threads per row with units of %u tiles do not fit one CTA for this "
                            "element type", threads_per_row, unit);
            p->tuned[segmented ? 1 : 0][size_class(n)] = static_cast<int8_t>(c);
            return GPS_OK;
        }
    }
    return fail(GPS_ERR_INVALID_ARGUMENT,
                "no launch configuration with %u tiles per unit, CTA divisor %u and %u threads per row", unit, ctas_div,
                threads_per_row);
}

gps_status gps_plan_generic_config(gps_plan p, int segmented, uint64_t n, uint32_t* out_unit, uint32_t* out_ctas_div,
                                   uint32_t* out_threads_per_row, int* out_tuned) {
    if (p == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "plan is NULL");
    const gps::GenericConfig cfg = generic_config(p, segmented != 0, n);
    if (out_unit) *out_unit = cfg.unit;
    if (out_ctas_div) *out_ctas_div = cfg.ctas_div;
    if (out_threads_per_row) *out_threads_per_row = cfg.split;
    if (out_tuned) *out_tuned = p->tuned[segmented ? 1 : 0][size_class(n)] >= 0 ? 1 : 0;
    return GPS_OK;
}

gps_status gps_select_flagged(gps_plan p, const void* d_in, const uint8_t* d_flags, void* d_out, uint64_t n,
                              uint64_t* d_num_selected, gps_stream_t stream) {
    if (p == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (p->algo != GPS_ALGO_CSDL) return fail(GPS_ERR_UNSUPPORTED, "select runs on chained-scan plans (GPS_ALGO_CSDL)");
    if (p->dtype == GPS_DTYPE_U32X4) return fail(GPS_ERR_UNSUPPORTED, "select takes 4- or 8-byte elements");
    if (d_num_selected == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "NULL count pointer");
    if ((reinterpret_cast<uintptr_t>(d_num_selected) & 7u) != 0)
        return fail(GPS_ERR_INVALID_ARGUMENT, "the count must be 8-byte aligned");
    gps_status st = check_device(p);
    if (st != GPS_OK) return st;
    const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (n == 0) {
        const cudaError_t err = cudaMemsetAsync(d_num_selected, 0, sizeof(uint64_t), s);
        return err == cudaSuccess ? GPS_OK : cuda_fail(err, "clearing the count");
    }
    if (n > p->max_n)
        return fail(GPS_ERR_SIZE_EXCEEDS_PLAN, "requested size %llu exceeds the plan's maximum %llu",
                    static_cast<unsigned long long>(n), static_cast<unsigned long long>(p->max_n));
    if (d_in == nullptr || d_flags == nullptr || d_out == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "NULL pointer");
    const size_t es = gps::dtype_size(p->dtype);
    const uintptr_t i = reinterpret_cast<uintptr_t>(d_in), fl = reinterpret_cast<uintptr_t>(d_flags);
    const uintptr_t o = reinterpret_cast<uintptr_t>(d_out);
    if (((i | fl) & 15u) != 0) return fail(GPS_ERR_INVALID_ARGUMENT, "values and flags must be 16-byte aligned");
    if ((o & (es - 1)) != 0) return fail(GPS_ERR_INVALID_ARGUMENT, "output must be aligned to the element size");
    const uint64_t bytes = n * es;
    if ((o < i + bytes && i < o + bytes) || (o < fl + n && fl < o + bytes))
        return fail(GPS_ERR_INVALID_ARGUMENT, "the output overlaps the values or the flags");
    if ((reinterpret_cast<uintptr_t>(p->desc16) & 15u) != 0)
        return fail(GPS_ERR_CUDA, "internal: misaligned descriptor region");
    gps::ScanArgs a{};
    a.in = d_in;
    a.out = d_out;
    a.n = n;
    a.num_tiles = static_cast<uint32_t>((n + gps::select_tile_elems(es) - 1) / gps::select_tile_elems(es));
    a.hdr = p->hdr16;
    a.desc = p->desc16;
    a.carry_out = d_num_selected;
    a.wait_budget_ns = p->wait_budget_ns;
    const cudaError_t err = gps::launch_select(es, a, d_flags, p->num_sms, s, &p->last_launch);
    if (err != cudaSuccess) return cuda_fail(err, "select launch");
    return GPS_OK;
}

gps_status gps_scan_host(gps_plan p, gps_scan_kind kind, const void* h_in, void* h_out, uint64_t n,
                         gps_stream_t stream) {
    if (p == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (!valid_kind(kind)) return fail(GPS_ERR_INVALID_ARGUMENT, "unknown scan kind %d", static_cast<int>(kind));
    if (n == 0) return GPS_OK;
    if (h_in == nullptr || h_out == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "NULL data pointer");
    if (generic_only(p->dtype)) return fail(GPS_ERR_UNSUPPORTED, "host-array scans take u32 and u64 plans");
    gps_status st = check_device(p);
    if (st != GPS_OK) return st;
    const size_t es = gps::dtype_size(p->dtype);
    cudaError_t err = cudaSuccess;
    if (p->stage[0] == nullptr) {
        // Chunk: up to kHostChunkBytes, whole tiles, within the plan's size.
        uint64_t chunk = std::min<uint64_t>(p->max_n, kHostChunkBytes / es);
        if (chunk > p->tile_elems) chunk -= chunk % p->tile_elems;
        for (int b = 0; b < kHostStages && err == cudaSuccess; ++b) err = cudaMalloc(&p->stage[b], chunk * es);
        if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&p->copy_in, cudaStreamNonBlocking);
        if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&p->compute, cudaStreamNonBlocking);
        if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&p->copy_out, cudaStreamNonBlocking);
        for (int b = 0; b < kHostStages && err == cudaSuccess; ++b) {
            err = cudaEventCreateWithFlags(&p->ev_loaded[b], cudaEventDisableTiming);
            if (err == cudaSuccess) err = cudaEventCreateWithFlags(&p->ev_scanned[b], cudaEventDisableTiming);
            if (err == cudaSuccess) err = cudaEventCreateWithFlags(&p->ev_free[b], cudaEventDisableTiming);
        }
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(&p->ev_start, cudaEventDisableTiming);
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(&p->ev_done, cudaEventDisableTiming);
        if (err != cudaSuccess) return cuda_fail(err, "host-scan staging setup");
        p->stage_elems = chunk;
    }
    cudaStream_t user = reinterpret_cast<cudaStream_t>(stream);
    const bool inclusive = kind == GPS_SCAN_INCLUSIVE;
    char* carry = static_cast<char*>(p->carries);
    // Work queued on the user's stream before this call comes first.
    err = cudaEventRecord(p->ev_start, user);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(p->copy_in, p->ev_start, 0);
    const uint64_t chunks = (n + p->stage_elems - 1) / p->stage_elems;
    for (uint64_t k = 0; k < chunks && err == cudaSuccess; ++k) {
        const int b = static_cast<int>(k % kHostStages);
        const uint64_t off = k * p->stage_elems;
        const uint64_t cnt = std::min<uint64_t>(p->stage_elems, n - off);
        if (k >= kHostStages) err = cudaStreamWaitEvent(p->copy_in, p->ev_free[b], 0);
        if (err == cudaSuccess)
            err = cudaMemcpyAsync(p->stage[b], static_cast<const char*>(h_in) + off * es, cnt * es,
                                  cudaMemcpyHostToDevice, p->copy_in);
        if (err == cudaSuccess) err = cudaEventRecord(p->ev_loaded[b], p->copy_in);
        if (err == cudaSuccess) err = cudaStreamWaitEvent(p->compute, p->ev_loaded[b], 0);
        if (err != cudaSuccess) break;
        const void* cin = k == 0 ? nullptr : carry + ((k - 1) & 1) * 64;
        void* cout = carry + (k & 1) * 64;
        st = launch_scan(p, inclusive, p->stage[b], p->stage[b], cnt, cin, cout, p->compute);
        if (st != GPS_OK) return st;
        err = cudaEventRecord(p->ev_scanned[b], p->compute);
        if (err == cudaSuccess) err = cudaStreamWaitEvent(p->copy_out, p->ev_scanned[b], 0);
        if (err == cudaSuccess)
            err = cudaMemcpyAsync(static_cast<char*>(h_out) + off * es, p->stage[b], cnt * es, cudaMemcpyDeviceToHost,
                                  p->copy_out);
        if (err == cudaSuccess) err = cudaEventRecord(p->ev_free[b], p->copy_out);
    }
    if (err == cudaSuccess) err = cudaEventRecord(p->ev_done, p->copy_out);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(user, p->ev_done, 0);
    if (err == cudaSuccess) err = cudaStreamSynchronize(user);
    if (err != cudaSuccess) return cuda_fail(err, "host-array scan");
    return GPS_OK;
}

gps_status gps_plan_check(gps_plan p, gps_stream_t stream) {
    if (p == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "plan is NULL");
    cudaError_t err = cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream));
    if (err != cudaSuccess) return cuda_fail(err, "cudaStreamSynchronize");
    uint32_t all = 0;
    for (gps::WsHeader* h : {p->hdr, p->hdr16}) {
        if (h == p->hdr16 && h == p->hdr) break;
        uint32_t flags = 0;
        err = cudaMemcpy(&flags, &h->error_flags, sizeof(flags), cudaMemcpyDeviceToHost);
        if (err != cudaSuccess) return cuda_fail(err, "reading device error flags");
        if (flags != 0) {
            const uint32_t zero = 0;
            err = cudaMemcpy(&h->error_flags, &zero, sizeof(zero), cudaMemcpyHostToDevice);
            if (err != cudaSuccess) return cuda_fail(err, "clearing device error flags");
        }
        all |= flags;
    }
    if (all != 0) return fail(GPS_ERR_TIMEOUT, "a device-side wait exceeded its budget (flags 0x%x)", all);
    return GPS_OK;
}

gps_status gps_plan_set_wait_budget(gps_plan p, uint64_t budget_ns) {
    if (p == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (budget_ns == 0) return fail(GPS_ERR_INVALID_ARGUMENT, "budget must be positive");
    p->wait_budget_ns = budget_ns;
    return GPS_OK;
}

gps_status gps_plan_set_stall(gps_plan p, uint32_t mode, uint32_t period, uint32_t seed, uint32_t delay_ns,
                              uint32_t fallback_polls) {
    if (p == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (mode > 2) return fail(GPS_ERR_INVALID_ARGUMENT, "unknown stall mode %u", mode);
    if (mode != 0 && p->algo != GPS_ALGO_CSDL)
        return fail(GPS_ERR_UNSUPPORTED, "forced-stall mode applies to the chained scan only");
    if (mode != 0 && period == 0) return fail(GPS_ERR_INVALID_ARGUMENT, "period must be positive");
    if (delay_ns > 1000000000u) return fail(GPS_ERR_INVALID_ARGUMENT, "delay %u ns exceeds one second", delay_ns);
    p->stall = gps::StallConfig{mode, period, seed, delay_ns, fallback_polls, 0};
    return GPS_OK;
}

gps_status gps_plan_set_fallback(gps_plan p, uint32_t fallback_polls) {
    if (p == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (fallback_polls != 0 && p->algo != GPS_ALGO_CSDL)
        return fail(GPS_ERR_UNSUPPORTED, "the decoupled fallback applies to the chained scan only");
    p->stall = gps::StallConfig{0, 1, 0, 0, fallback_polls, 0};
    return GPS_OK;
}

gps_status gps_plan_stats(gps_plan p, gps_stream_t stream, gps_lookback_stats* out) {
    if (p == nullptr || out == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "NULL argument");
    cudaError_t err = cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream));
    gps::WsHeader h{};
    if (err == cudaSuccess) err = cudaMemcpy(&h, p->hdr, sizeof(h), cudaMemcpyDeviceToHost);
    if (err != cudaSuccess) return cuda_fail(err, "reading statistics");
    out->polls = h.stat_polls;
    out->fallbacks = h.stat_fallbacks;
    out->inserts = h.stat_inserts;
    out->stalls = h.stat_stalls;
    return GPS_OK;
}

gps_status gps_plan_geometry(gps_plan p, uint64_t n, uint32_t* tile_elems, uint32_t* grid, uint32_t* launches) {
    if (p == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (tile_elems) *tile_elems = p->tile_elems;
    if (grid) *grid = static_cast<uint32_t>(p->last_launch.grid);
    const bool small = !generic_only(p->dtype) && n <= p->small_max && p->stall.mode == 0 && p->stall.fallback_polls == 0;
    if (launches) *launches = n == 0 ? 0u : (small || p->algo == GPS_ALGO_CSDL ? 1u : 3u);
    return GPS_OK;
}

gps_status gps_plan_set_mid_max(gps_plan p, uint64_t max_n) {
    if (p == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (max_n != 0 && (p->algo != GPS_ALGO_CSDL || generic_only(p->dtype)))
        return fail(GPS_ERR_UNSUPPORTED, "the one-tile-per-CTA scan runs integer chained-scan plans only");
    p->mid_max = max_n;
    return GPS_OK;
}

gps_status gps_plan_set_small_max(gps_plan p, uint64_t max_n) {
    if (p == nullptr) return fail(GPS_ERR_INVALID_ARGUMENT, "plan is NULL");
    const uint64_t cap = gps::small_scan_max_elems(p->dtype);
    if (max_n > cap)
        return fail(GPS_ERR_INVALID_ARGUMENT, "the one-CTA scan takes at most %llu elements of this type",
                    static_cast<unsigned long long>(cap));
    p->small_max = max_n;
    return GPS_OK;
}

}  // extern "C"
