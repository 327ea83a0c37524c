// Chained scan of uint32 elements that allocates no memory.
//
// gps_scan() needs a plan, and gps_plan_create() calls cudaMalloc. Some
// callers cannot do that: code that runs under a fixed device-memory budget
// set up by its host application, code called from a context where the
// allocator must not be entered (for example from inside another library's
// allocation or stream callbacks), or latency-critical code that may not pay
// for cudaMalloc's implicit synchronisation. For them, gps_scan_u32_noalloc()
// runs the same chained-scan kernels with their scratch memory (the
// workspace header and the tile descriptors) in a fixed array of this file,
// which the CUDA module holds on every device that loads the library, until
// the process exits.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <mutex>

#include "gps_internal.h"
#include "launch_util.h"

namespace {

// Largest scan this entry point accepts, and the scratch it needs: the
// workspace header, the two carry slots the plan layout reserves, and one
// descriptor per 4096-element tile plus the lookback padding -- the same
// sizing rule gps_plan_create() uses for a chained-scan plan of this size.
constexpr uint64_t kMaxN = 1ull << 28;
constexpr uint64_t kTileElems = 4096;
constexpr size_t kHeaderBytes = sizeof(gps::WsHeader);
constexpr size_t kCarryBytes = 128;
constexpr uint64_t kMaxTiles = (kMaxN + kTileElems - 1) / kTileElems;
constexpr size_t kDescSlots = kMaxTiles + gps::kDescPad;
constexpr size_t kScratchBytes = kHeaderBytes + kCarryBytes + kDescSlots * sizeof(uint64_t);

// The scratch itself. In host code this name is only a stand-in for the
// device address; the kernels get the address from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;

// Set-up of one device, valid for the driver context it was made in. The
// device address of the array belongs to the context that loaded the module:
// after cudaDeviceReset(), or when the caller makes another driver context
// current on the same device, the array lives at another address. The
// context's id (cuCtxGetId) is unique for the life of the process, so a
// cached address is used only in the context that produced it.
struct DeviceSetup {
    unsigned long long ctx_id;  // 0: not set up
    void* scratch;              // device address of g_noalloc_scratch in that context
    int num_sms;
};

std::mutex g_setup_mu;
DeviceSetup g_setup[kMaxDevices];

gps_status reject(gps_status st, const char* msg) {
    gps::record_error(msg);
    return st;
}

}  // namespace

extern "C" {

gps_status gps_scan_u32_noalloc(gps_scan_kind kind, const void* d_in, void* d_out, uint64_t n,
                                gps_stream_t stream) {
    static_assert(kMaxN == GPS_NOALLOC_MAX_N, "the header states the same limit");
    if (kind != GPS_SCAN_EXCLUSIVE && kind != GPS_SCAN_INCLUSIVE)
        return reject(GPS_ERR_INVALID_ARGUMENT, "unknown scan kind");
    if (n == 0) return GPS_OK;
    if (n > kMaxN)
        return reject(GPS_ERR_SIZE_EXCEEDS_PLAN,
                      "gps_scan_u32_noalloc: n exceeds GPS_NOALLOC_MAX_N (2^28 elements); use a plan for larger scans");
    if (d_in == nullptr || d_out == nullptr) return reject(GPS_ERR_INVALID_ARGUMENT, "NULL data pointer");
    const uintptr_t i = reinterpret_cast<uintptr_t>(d_in), o = reinterpret_cast<uintptr_t>(d_out);
    if ((i % 4) != 0 || (o % 4) != 0)
        return reject(GPS_ERR_INVALID_ARGUMENT, "pointers must be aligned to the 4-byte element size");
    const uint64_t bytes = n * 4;
    if (i != o && i < o + bytes && o < i + bytes)
        return reject(GPS_ERR_INVALID_ARGUMENT, "input and output overlap without being identical");
    if (gps::csdl_tile_elems(GPS_DTYPE_U32) != kTileElems)
        return reject(GPS_ERR_UNSUPPORTED, "gps_scan_u32_noalloc: scratch sized for a different tile size");

    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return reject(GPS_ERR_CUDA, "gps_scan_u32_noalloc: no usable current device");
    DeviceSetup setup;
    {
        // First call on this device in the current context: look up the
        // scratch array's device address and the SM count with this device
        // current, and set up the launch attributes of every kernel variant
        // this entry point can launch, so that later calls (possibly inside a
        // stream capture) query nothing.
        std::lock_guard<std::mutex> lock(g_setup_mu);
        unsigned long long ctx = gps::current_ctx_id();
        if (ctx == 0 || g_setup[dev].ctx_id != ctx) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr)
                return reject(GPS_ERR_CUDA, "gps_scan_u32_noalloc: cudaGetSymbolAddress of the scratch array failed");
            int sms = 0;
            if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
                return reject(GPS_ERR_CUDA, "gps_scan_u32_noalloc: device query failed");
            if (gps::prepare_csdl(GPS_DTYPE_U32) != cudaSuccess)
                return reject(GPS_ERR_CUDA, "gps_scan_u32_noalloc: kernel set-up failed");
            // cudaGetSymbolAddress has made the primary context current if no
            // context was.
            if (ctx == 0) ctx = gps::current_ctx_id();
            if (ctx == 0) return reject(GPS_ERR_CUDA, "gps_scan_u32_noalloc: no current CUDA context");
            g_setup[dev] = DeviceSetup{ctx, p, sms};
        }
        setup = g_setup[dev];
    }

    // The array keeps what the previous call left: zero the header and the
    // descriptors this scan uses (a stale descriptor must read "not ready").
    const uint64_t tiles = (n + kTileElems - 1) / kTileElems;
    const size_t used = kHeaderBytes + kCarryBytes + (tiles + gps::kDescPad) * sizeof(uint64_t);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(setup.scratch, 0, used, st) != cudaSuccess)
        return reject(GPS_ERR_CUDA, "gps_scan_u32_noalloc: clearing the scratch failed");

    gps::ScanArgs a{};
    a.in = d_in;
    a.out = d_out;
    a.n = n;
    a.num_tiles = static_cast<uint32_t>(tiles);
    a.hdr = static_cast<gps::WsHeader*>(setup.scratch);
    a.desc = static_cast<char*>(setup.scratch) + kHeaderBytes + kCarryBytes;
    a.wait_budget_ns = 1000000000ull;
    if (gps::launch_csdl(GPS_DTYPE_U32, kind == GPS_SCAN_INCLUSIVE, false, a, setup.num_sms, st, nullptr) !=
        cudaSuccess)
        return reject(GPS_ERR_CUDA, "gps_scan_u32_noalloc: kernel launch failed");
    return GPS_OK;
}

}  // extern "C"
