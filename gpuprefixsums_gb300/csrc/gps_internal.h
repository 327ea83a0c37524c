// Internal definitions shared by the scan kernels and the C ABI layer:
// the device workspace header, the tile-descriptor encodings and the kernel
// argument block.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

#include "gps.h"

namespace gps {

// Tile ids handed out by the producer; kTileEnd marks "no more tiles".
constexpr uint32_t kTileEnd = 0xFFFFFFFFu;

// Epochs are 30 bits wide so that they fit beside a 32-bit value in a 64-bit
// descriptor. Epoch 0 never occurs, so a zeroed workspace is "not ready".
constexpr uint32_t kEpochMask = 0x3FFFFFFFu;

// Descriptor slots allocated past the last tile: a lookback window is read in
// aligned groups of up to 16 slots and may end up to 15 slots after its tile.
constexpr uint32_t kDescPad = 16;

// Descriptor status (two bits), as in the decoupled-lookback scheme:
// not ready / tile aggregate only / inclusive prefix through this tile.
enum DescStatus : uint32_t { kNotReady = 0, kAggregate = 1, kInclusive = 2 };

// Bits of WsHeader::error_flags.
enum ErrFlag : uint32_t {
    kErrLookbackTimeout = 1u,  // a lookback spin ran past its wait budget
    kErrPipelineTimeout = 2u,  // an mbarrier wait ran past its wait budget
    kErrStallTimeout = 4u,     // a forced-stall wait ran past its wait budget
};

// Device-resident state of one plan. Zeroed at plan creation, then epoch=1.
// tile_counter / exit_counter are returned to zero by the last CTA of every
// launch, and the same CTA advances the epoch, so consecutive launches need no
// memset and a launch can be replayed from a CUDA graph.
struct alignas(128) WsHeader {
    uint32_t tile_counter;
    uint32_t exit_counter;
    uint32_t epoch;
    uint32_t error_flags;
    unsigned long long capacity_tiles;  // descriptor slots that follow
    unsigned long long stat_polls;      // lookback windows re-polled (stats mode)
    unsigned long long stat_fallbacks;  // predecessor tiles re-reduced
    unsigned long long stat_inserts;    // fallback aggregates that won the CAS
    unsigned long long stat_stalls;     // tiles that were made to stall
};
static_assert(sizeof(WsHeader) == 128, "header is one 128-byte line");

// Forced-stall test mode (EmulatedDeadlocking-style).
//  mode 0: off.
//  mode 1: every tile with (t % period) == 0 stalls (the reference pattern).
//  mode 2: tiles selected by a seeded hash with probability 1/period stall.
// A stalled tile withholds its aggregate for up to delay_ns or until a
// successor re-reduces its input and inserts the aggregate for it
// (fallback_polls > 0 enables that fallback after this many empty polls).
struct StallConfig {
    uint32_t mode;
    uint32_t period;
    uint32_t seed;
    uint32_t delay_ns;
    uint32_t fallback_polls;
    uint32_t pad_;
};

enum class PrefixMode : int { Lookback = 0, Spine = 1 };

// Fixed-order lookback of the generic kernel (scan_seg.cuh): lookback units
// per group, and the group descriptors a plan keeps for up to `units` units
// (one more than the groups, as slack).
constexpr uint32_t kDetGroupUnits = 128;
constexpr uint64_t det_group_slots(uint64_t units) { return (units + kDetGroupUnits - 1) / kDetGroupUnits + 1; }

// The generic kernel's unit and group descriptors sit one per 128-byte line
// (a stride of 8 words) when a launch has at most kSegStrideMaxUnits
// lookback units, else packed (Op::kDescWords words each). Measured on GB300
// (FP32, GPU time per scan): one per line 11.6 against 12.4 us at 2^20, 14.9
// against 15.7 at 2^22, 29.0 against 31.7 at 2^24 (1024 units of 4 tiles);
// packed 91 against 94 us at 2^26 and 173 against 178 at 2^27, where the
// wider reads compete with the data for L2. 16-byte words a plan keeps for
// up to `tiles` units of `dw` words, and for their group descriptors:
constexpr uint32_t kSegDescStride = 8;
constexpr uint64_t kSegStrideMaxUnits = 1024;
constexpr uint64_t seg_desc_words(uint64_t tiles, uint64_t dw) {
    const uint64_t packed = (tiles + kDescPad) * dw;
    const uint64_t strided = ((tiles < kSegStrideMaxUnits ? tiles : kSegStrideMaxUnits) + kDescPad) * kSegDescStride;
    return packed > strided ? packed : strided;
}
constexpr uint64_t seg_group_words(uint64_t tiles, uint64_t dw) {
    const uint64_t packed = det_group_slots(tiles) * dw;
    const uint64_t strided = det_group_slots(tiles < kSegStrideMaxUnits ? tiles : kSegStrideMaxUnits) * kSegDescStride;
    return packed > strided ? packed : strided;
}

struct ScanArgs {
    const void* in;
    void* out;
    uint64_t n;
    uint32_t num_tiles;
    // One-tile-per-CTA and generic kernels: 16-byte words from one descriptor
    // to the next (0: packed), set by their launchers.
    uint32_t desc_stride;
    WsHeader* hdr;       // plan state (counters, epoch, error flags)
    void* desc;          // tile descriptors (lookback)
    // Descriptors of groups: of 32 tiles for the one-tile-per-CTA kernels, of
    // kDetGroupUnits lookback units for the generic kernel.
    void* group_desc;
    const void* spine;   // inclusive scan of tile sums (reduce-then-scan)
    const void* carry_in;  // optional: one element added to every output
    void* carry_out;       // optional: receives carry_in + sum of all n inputs
    uint64_t wait_budget_ns;
    StallConfig stall;
};

// Kernel geometry shared by host and device: RW reduce warps and RW finalize
// warps, each thread of either owning 128 contiguous bytes of the tile, plus
// one producer warp and kLookbackWarps lookback warps per CTA.
template <typename T, int RW>
struct TileShape {
    static constexpr int kItems = 128 / static_cast<int>(sizeof(T));
    static constexpr int kRoleThreads = RW * 32;
    static constexpr int kTile = kRoleThreads * kItems;
    static constexpr int kLookbackWarps = 2;
    static constexpr int kThreads = 32 * (1 + kLookbackWarps + 2 * RW);
};

// Segments of a batched (segmented) scan: segment s is
// [offsets[s], offsets[s+1]); offsets has num_segments + 1 entries.
struct SegArgs {
    const uint32_t* offsets;
    uint32_t num_segments;
};

// ------------------------------------------------------------ launchers
// Each returns the launch status; they never synchronize.
struct LaunchInfo {
    int grid;
    int block;
    size_t smem;
};

cudaError_t launch_csdl(gps_dtype dtype, bool inclusive, bool stall_mode, const ScanArgs& a,
                        int num_sms, cudaStream_t stream, LaunchInfo* info);
// Sets up, without launching, every kernel launch_csdl() can pick for this
// dtype without forced stalls, so that later launches make no set-up call.
cudaError_t prepare_csdl(gps_dtype dtype);
cudaError_t launch_rts(gps_dtype dtype, bool inclusive, const ScanArgs& a, void* tile_sums,
                       int num_sms, cudaStream_t stream, LaunchInfo* info);
// Tensor maps of the generic kernel: the buffer seen as rows of 128 bytes
// (32 four-byte or 16 eight-byte elements), boxes of 128 rows (one 16 KB
// tile), 128-byte swizzle. Rows past the last full row are the kernel's to
// handle with plain loads and stores. Host-side; encodes through the driver
// entry point cuTensorMapEncodeTiled.
struct RowMaps {
    CUtensorMap in;
    CUtensorMap out;
};
cudaError_t encode_row_maps(const void* in, void* out, uint64_t n, uint32_t elem_size, RowMaps* maps);

// Launch configuration of the generic kernel: tiles per lookback unit (1 or
// 4; the unit is what one CTA takes from the work counter), the CTA count as
// a fraction of the resident maximum (1 = all, 2 = half), and threads per
// 128-byte row of a tile (1: 4 reduce and 4 finalize warps, each thread
// scanning 128 bytes; 2: 8 and 8, each thread scanning 64 bytes).
struct GenericConfig {
    uint32_t unit;
    uint32_t ctas_div;
    uint32_t split;
};
constexpr GenericConfig kGenericCandidates[] = {{4, 1, 1}, {1, 1, 1}, {4, 2, 1}, {1, 2, 1},
                                                {4, 1, 2}, {1, 1, 2}, {4, 2, 2}, {1, 2, 2}};
constexpr int kNumGenericCandidates = 8;
// Untuned choice: units of 4 tiles once there are at least two such units
// per SM, else single-tile units (more CTAs busy on small inputs).
GenericConfig default_generic_config(uint64_t n, uint32_t tile_elems, int num_sms);

// Generic single-pass scan (scan_seg.cuh), one per scan operation; `sg` null
// for a plain scan. Buffers must be 16-byte aligned; descriptors are 16 bytes.
cudaError_t launch_seg_u32(bool inclusive, const ScanArgs& a, const SegArgs* sg, const GenericConfig& cfg, int num_sms,
                           cudaStream_t stream, LaunchInfo* info);
cudaError_t launch_seg_u64(bool inclusive, const ScanArgs& a, const SegArgs* sg, const GenericConfig& cfg, int num_sms,
                           cudaStream_t stream, LaunchInfo* info);
cudaError_t launch_seg_f32(bool inclusive, const ScanArgs& a, const SegArgs* sg, const GenericConfig& cfg, int num_sms,
                           cudaStream_t stream, LaunchInfo* info);
cudaError_t launch_seg_f32c(bool inclusive, const ScanArgs& a, const SegArgs* sg, const GenericConfig& cfg,
                            int num_sms, cudaStream_t stream, LaunchInfo* info);
cudaError_t launch_seg_u32x4(bool inclusive, const ScanArgs& a, const SegArgs* sg, const GenericConfig& cfg,
                             int num_sms, cudaStream_t stream, LaunchInfo* info);
// The same with two threads per row (cfg.split == 2), in translation units of
// their own (seg_*_x2.cu); cudaErrorNotSupported when that kernel shape does
// not fit one CTA's shared memory for the type.
cudaError_t launch_seg_u32_x2(bool inclusive, const ScanArgs& a, const SegArgs* sg, const GenericConfig& cfg,
                              int num_sms, cudaStream_t stream, LaunchInfo* info);
cudaError_t launch_seg_u64_x2(bool inclusive, const ScanArgs& a, const SegArgs* sg, const GenericConfig& cfg,
                              int num_sms, cudaStream_t stream, LaunchInfo* info);
cudaError_t launch_seg_f32_x2(bool inclusive, const ScanArgs& a, const SegArgs* sg, const GenericConfig& cfg,
                              int num_sms, cudaStream_t stream, LaunchInfo* info);
cudaError_t launch_seg_f32c_x2(bool inclusive, const ScanArgs& a, const SegArgs* sg, const GenericConfig& cfg,
                               int num_sms, cudaStream_t stream, LaunchInfo* info);
cudaError_t launch_seg_u32x4_x2(bool inclusive, const ScanArgs& a, const SegArgs* sg, const GenericConfig& cfg,
                                int num_sms, cudaStream_t stream, LaunchInfo* info);
// Whether the two-threads-per-row kernels of a unit size fit one CTA.
bool seg_u32_x2_fits(uint32_t unit);
bool seg_u64_x2_fits(uint32_t unit);
bool seg_f32_x2_fits(uint32_t unit);
bool seg_f32c_x2_fits(uint32_t unit);
bool seg_u32x4_x2_fits(uint32_t unit);

// Stream compaction by flag bytes (select.cu): elements per tile for an
// element size, and the launch. a.carry_out receives the count (uint64).
uint32_t select_tile_elems(size_t elem_size);
cudaError_t launch_select(size_t elem_size, const ScanArgs& a, const uint8_t* flags, int num_sms, cudaStream_t stream,
                          LaunchInfo* info);

// Small integer scans in one CTA (small.cu): up to kSmallMaxBytes of input.
constexpr size_t kSmallMaxBytes = 64 * 1024;
uint64_t small_scan_max_elems(gps_dtype dtype);
cudaError_t launch_small(gps_dtype dtype, bool inclusive, const ScanArgs& a, cudaStream_t stream, LaunchInfo* info);

// Integer chained scans up to mid size, one 16 KB tile per CTA (mid.cu); the
// default upper size of a plan, in bytes of input. Measured on GB300 (graph
// replay; descriptors one per line): one tile per CTA is faster than the
// persistent kernel up to 64 MB (u32: 31.8 against 34.4 us at 2^24; u64:
// 32.1 against 32.8 us at 2^23), slower from 96 MB (u32: 43.7 against 44.6
// us at 3 x 2^23 at best, 56.5 against 53.7 at 2^25; u64: 44.5 against 43.2
// at 3 x 2^22).
constexpr size_t kMidMaxBytes = 64ull << 20;
// Tile descriptors of the one-tile-per-CTA kernels sit one per 128-byte line
// (a stride of 8 words) when a launch has more than one group of 32 tiles
// and at most kMidStrideMaxTiles tiles, else packed. Sharing lines between
// tiles that publish and read at the same moment cost up to 3 us per read
// (2^20 u32: 6.04 us packed, 4.95 us one per line, 5.23 us one per 32-byte
// sector); with one group, packed reads are faster (2^17: 2.83 against
// 3.36 us). Group descriptors always take a line each (2^22 u32: 7.56
// against 8.84 us packed). Tile-descriptor words a plan keeps for `tiles`
// tiles:
constexpr uint32_t kMidDescStride = 8;
constexpr uint64_t kMidStrideMaxTiles = 4096;
constexpr uint64_t mid_desc_words(uint64_t tiles) {
    const uint64_t strided = ((tiles < kMidStrideMaxTiles ? tiles : kMidStrideMaxTiles) + kDescPad) * kMidDescStride;
    return tiles + kDescPad > strided ? tiles + kDescPad : strided;
}
cudaError_t launch_mid(gps_dtype dtype, bool inclusive, const ScanArgs& a, int num_sms, cudaStream_t stream,
                       LaunchInfo* info);

uint32_t csdl_tile_elems(gps_dtype dtype);
// Sets the text gps_last_error() returns on this host thread.
void record_error(const char* msg);
uint32_t rts_tile_elems(gps_dtype dtype);
size_t dtype_size(gps_dtype dtype);

}  // namespace gps
