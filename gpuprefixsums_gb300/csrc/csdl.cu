// Chained scan with decoupled lookback (single pass) for u32 and u64.
// Drop-in for ChainedScanDecoupledLookback::CSDLExclusive / CSDLInclusive
// (GPUPrefixSumsCUDA/ChainedScanDecoupledLookback.cuh:141-153) as launched by
// ChainedScanDecoupledLookbackDispatcher::DispatchKernels{Ex,In}clusive
// (ChainedScanDecoupledLookbackDispatcher.cuh:177-195). The reference clears
// its descriptors and bump counter with two cudaMemsets per call; here the
// kernel leaves its workspace ready for the next launch itself.
#include "launch_util.h"
#include "scan_l2.cuh"
#include "scan_pipeline.cuh"

namespace gps {

namespace {

// Shape: 4 reduce + 4 finalize warps over 16 KB tiles (4096 u32 / 2048 u64),
// a 12-deep ring (192 KB of shared memory, one CTA per SM) holding three
// lookback units of 4 tiles (64 KB) each. One CTA per SM and 64 KB units keep
// the number of descriptors every lookback reads, and the number of readers,
// small.
constexpr int kCsdlWarps = 4;
constexpr int kCsdlStages = 12;
constexpr int kCsdlUnit = 4;  // tiles per lookback unit

template <typename T, bool INCL, bool BULK, bool STALL>
cudaError_t launch_csdl_t(const ScanArgs& a, int num_sms, cudaStream_t stream, LaunchInfo* info) {
    using Shape = TileShape<T, kCsdlWarps>;
    auto kern = scan_pipeline_kernel<T, kCsdlWarps, kCsdlStages, kCsdlUnit, INCL, BULK, PrefixMode::Lookback, STALL>;
    constexpr size_t smem = pipeline_smem_bytes<T, kCsdlWarps, kCsdlStages>();
    int occ = 0;
    cudaError_t err = resident_ctas_per_sm(kern, Shape::kThreads, smem, &occ);
    if (err != cudaSuccess) return err;
    const int grid = persistent_grid(a.num_tiles, occ, num_sms);
    if (info) *info = LaunchInfo{grid, Shape::kThreads, smem};
    kern<<<grid, Shape::kThreads, smem, stream>>>(a);
    return cudaGetLastError();
}

// L2-buffered kernel (16-byte-aligned buffers): 4 reduce + 4 finalize warps
// over 16 KB tiles, lookback units of 4 tiles (64 KB), 6 units in flight per
// CTA, one CTA per SM. Each unit is prefetched into L2 when its id is taken,
// so the reduce-pass ring needs few stages: 4 reduce-pass and 9 scan-pass
// stages (208 KB; 3 + 9 for u64, whose per-thread prefixes take twice the
// room). Measured on GB300 at 2^28 u32 elements: 4 + 9 stages beat 5 + 8 by
// 4% once the prefetch was in (3 + 10 starves the reduce pass), and 6 units
// in flight beat 4, 5 and 7 (the queue depth sets how much input waits in L2
// between the two passes, 152 x 6 x 64 KB at most).
constexpr int kL2Warps = 4;
template <typename T>
constexpr int kL2RStages = sizeof(T) == 8 ? 3 : 4;
constexpr int kL2SStages = 9;
constexpr int kL2Queue = 6;
constexpr int kL2Unit = 4;

template <typename T, bool INCL, bool STALL>
cudaError_t launch_l2_t(const ScanArgs& a, int num_sms, cudaStream_t stream, LaunchInfo* info) {
    auto kern = scan_l2_kernel<T, kL2Warps, kL2RStages<T>, kL2SStages, kL2Queue, kL2Unit, INCL, STALL>;
    constexpr size_t smem = l2_smem_bytes<T, kL2Warps, kL2RStages<T>, kL2SStages, kL2Queue, kL2Unit>();
    static_assert(smem <= 232448, "227 KB of shared memory per CTA");
    constexpr int threads = L2Shape<T, kL2Warps>::kThreads;
    int occ = 0;
    cudaError_t err = resident_ctas_per_sm(kern, threads, smem, &occ);
    if (err != cudaSuccess) return err;
    const uint32_t units = (a.num_tiles + kL2Unit - 1) / kL2Unit;
    const int grid = persistent_grid(units, occ, num_sms);
    if (info) *info = LaunchInfo{grid, threads, smem};
    kern<<<grid, threads, smem, stream>>>(a);
    return cudaGetLastError();
}

// Sets up (shared-memory opt-in, occupancy) the four kernels a chained scan
// without forced stalls can launch: exclusive and inclusive, bulk-copy and
// ring, without launching them.
template <typename T>
cudaError_t prepare_csdl_t() {
    int occ = 0;
    cudaError_t err = cudaSuccess;
    {
        constexpr size_t smem = l2_smem_bytes<T, kL2Warps, kL2RStages<T>, kL2SStages, kL2Queue, kL2Unit>();
        constexpr int threads = L2Shape<T, kL2Warps>::kThreads;
        err = resident_ctas_per_sm(scan_l2_kernel<T, kL2Warps, kL2RStages<T>, kL2SStages, kL2Queue, kL2Unit, false,
                                                  false>, threads, smem, &occ);
        if (err == cudaSuccess)
            err = resident_ctas_per_sm(scan_l2_kernel<T, kL2Warps, kL2RStages<T>, kL2SStages, kL2Queue, kL2Unit, true,
                                                      false>, threads, smem, &occ);
    }
    if (err == cudaSuccess) {
        using Shape = TileShape<T, kCsdlWarps>;
        constexpr size_t smem = pipeline_smem_bytes<T, kCsdlWarps, kCsdlStages>();
        err = resident_ctas_per_sm(scan_pipeline_kernel<T, kCsdlWarps, kCsdlStages, kCsdlUnit, false, false,
                                                        PrefixMode::Lookback, false>, Shape::kThreads, smem, &occ);
        if (err == cudaSuccess)
            err = resident_ctas_per_sm(scan_pipeline_kernel<T, kCsdlWarps, kCsdlStages, kCsdlUnit, true, false,
                                                            PrefixMode::Lookback, false>, Shape::kThreads, smem, &occ);
    }
    return err;
}

template <typename T>
cudaError_t dispatch_csdl(bool inclusive, bool stall, const ScanArgs& a, int num_sms, cudaStream_t stream,
                          LaunchInfo* info) {
    const bool bulk = ((reinterpret_cast<uintptr_t>(a.in) | reinterpret_cast<uintptr_t>(a.out)) & 15u) == 0;
    if (bulk) {
        if (stall)
            return inclusive ? launch_l2_t<T, true, true>(a, num_sms, stream, info)
                             : launch_l2_t<T, false, true>(a, num_sms, stream, info);
        return inclusive ? launch_l2_t<T, true, false>(a, num_sms, stream, info)
                         : launch_l2_t<T, false, false>(a, num_sms, stream, info);
    }
    // The forced-stall test mode wants aligned buffers; the fallback alone
    // (stall mode 0) is a robustness option the ring kernel runs without.
    if (stall && a.stall.mode != 0) return cudaErrorInvalidValue;
    return inclusive ? launch_csdl_t<T, true, false, false>(a, num_sms, stream, info)
                     : launch_csdl_t<T, false, false, false>(a, num_sms, stream, info);
}

}  // namespace

uint32_t csdl_tile_elems(gps_dtype dtype) {
    // Struct elements (16 bytes) run on the generic kernel's 16 KB tiles.
    if (dtype == GPS_DTYPE_U32X4) return 16384 / 16;
    return dtype == GPS_DTYPE_U64 ? TileShape<uint64_t, kCsdlWarps>::kTile : TileShape<uint32_t, kCsdlWarps>::kTile;
}

cudaError_t prepare_csdl(gps_dtype dtype) {
    return dtype == GPS_DTYPE_U64 ? prepare_csdl_t<uint64_t>() : prepare_csdl_t<uint32_t>();
}

cudaError_t launch_csdl(gps_dtype dtype, bool inclusive, bool stall_mode, const ScanArgs& a, int num_sms,
                        cudaStream_t stream, LaunchInfo* info) {
    if (dtype == GPS_DTYPE_U64) return dispatch_csdl<uint64_t>(inclusive, stall_mode, a, num_sms, stream, info);
    return dispatch_csdl<uint32_t>(inclusive, stall_mode, a, num_sms, stream, info);
}

}  // namespace gps
