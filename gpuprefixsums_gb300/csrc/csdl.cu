// Chained scan with decoupled lookback (single pass) for u32 and u64.
// Drop-in for ChainedScanDecoupledLookback::CSDLExclusive / CSDLInclusive
// (GPUPrefixSumsCUDA/ChainedScanDecoupledLookback.cuh:141-153) as launched by
// ChainedScanDecoupledLookbackDispatcher::DispatchKernels{Ex,In}clusive
// (ChainedScanDecoupledLookbackDispatcher.cuh:177-195). The reference clears
// its descriptors and bump counter with two cudaMemsets per call; here the
// kernel leaves its workspace ready for the next launch itself.
#include "launch_util.h"
#include "scan_pipeline.cuh"

namespace gps {

namespace {

// Tuned shape: 8 consumer warps, 4-deep ring of 16 KB tiles (64 KB of
// shared memory per CTA, 3 CTAs per SM).
constexpr int kCsdlWarps = 8;
constexpr int kCsdlStages = 4;

template <typename T, bool INCL, bool BULK, bool STALL>
cudaError_t launch_csdl_t(const ScanArgs& a, int num_sms, cudaStream_t stream, LaunchInfo* info) {
    using Shape = TileShape<T, kCsdlWarps>;
    auto kern = scan_pipeline_kernel<T, kCsdlWarps, kCsdlStages, INCL, BULK, PrefixMode::Lookback, STALL>;
    constexpr size_t smem = pipeline_smem_bytes<T, kCsdlWarps, kCsdlStages>();
    int occ = 0;
    cudaError_t err = resident_ctas_per_sm(kern, Shape::kThreads, smem, &occ);
    if (err != cudaSuccess) return err;
    const int grid = persistent_grid(a.num_tiles, occ, num_sms);
    if (info) *info = LaunchInfo{grid, Shape::kThreads, smem};
    kern<<<grid, Shape::kThreads, smem, stream>>>(a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t dispatch_csdl(bool inclusive, bool stall, const ScanArgs& a, int num_sms, cudaStream_t stream,
                          LaunchInfo* info) {
    const bool bulk = ((reinterpret_cast<uintptr_t>(a.in) | reinterpret_cast<uintptr_t>(a.out)) & 15u) == 0;
    if (stall) {
        if (!bulk) return cudaErrorInvalidValue;  // test mode wants aligned buffers
        return inclusive ? launch_csdl_t<T, true, true, true>(a, num_sms, stream, info)
                         : launch_csdl_t<T, false, true, true>(a, num_sms, stream, info);
    }
    if (bulk)
        return inclusive ? launch_csdl_t<T, true, true, false>(a, num_sms, stream, info)
                         : launch_csdl_t<T, false, true, false>(a, num_sms, stream, info);
    return inclusive ? launch_csdl_t<T, true, false, false>(a, num_sms, stream, info)
                     : launch_csdl_t<T, false, false, false>(a, num_sms, stream, info);
}

}  // namespace

uint32_t csdl_tile_elems(gps_dtype dtype) {
    return dtype == GPS_DTYPE_U64 ? TileShape<uint64_t, kCsdlWarps>::kTile : TileShape<uint32_t, kCsdlWarps>::kTile;
}

cudaError_t launch_csdl(gps_dtype dtype, bool inclusive, bool stall_mode, const ScanArgs& a, int num_sms,
                        cudaStream_t stream, LaunchInfo* info) {
    if (dtype == GPS_DTYPE_U64) return dispatch_csdl<uint64_t>(inclusive, stall_mode, a, num_sms, stream, info);
    return dispatch_csdl<uint32_t>(inclusive, stall_mode, a, num_sms, stream, info);
}

}  // namespace gps
