// Launcher of the generic kernel (scan_seg.cuh) for one scan operation;
// included by one .cu file per operation so that the instantiations compile
// in parallel.
#pragma once
#include "launch_util.h"
#include "scan_seg.cuh"

namespace gps {

// 4 reduce + 4 finalize warps over 16 KB tiles, 5 reduce-pass and 8
// scan-pass stages, units of 4 tiles, 6 units in flight per CTA (the
// measured optimum of the u32 L2-buffered kernel, scan_l2.cuh).
constexpr int kSegWarps = 4;
constexpr int kSegRStages = 5;
constexpr int kSegSStages = 8;
constexpr int kSegQueue = 6;
constexpr int kSegUnit = 4;

template <class Op, bool INCL, bool SEG>
cudaError_t launch_seg_t(const ScanArgs& a, const SegArgs& sg, int num_sms, cudaStream_t stream, LaunchInfo* info) {
    auto kern = scan_seg_kernel<Op, kSegWarps, kSegRStages, kSegSStages, kSegQueue, kSegUnit, INCL, SEG>;
    constexpr size_t smem = seg_smem_bytes<Op, kSegWarps, kSegRStages, kSegSStages, kSegQueue, kSegUnit, SEG>();
    static_assert(smem <= 232448, "227 KB of shared memory per CTA");
    constexpr int threads = SegShape<Op, kSegWarps>::kThreads;
    int occ = 0;
    cudaError_t err = resident_ctas_per_sm(kern, threads, smem, &occ);
    if (err != cudaSuccess) return err;
    const uint32_t units = (a.num_tiles + kSegUnit - 1) / kSegUnit;
    const int grid = persistent_grid(units, occ, num_sms);
    if (info) *info = LaunchInfo{grid, threads, smem};
    kern<<<grid, threads, smem, stream>>>(a, sg);
    return cudaGetLastError();
}

template <class Op>
cudaError_t launch_seg_op(bool inclusive, const ScanArgs& a, const SegArgs* sg, int num_sms, cudaStream_t stream,
                          LaunchInfo* info) {
    const SegArgs none{nullptr, 0};
    if (sg != nullptr)
        return inclusive ? launch_seg_t<Op, true, true>(a, *sg, num_sms, stream, info)
                         : launch_seg_t<Op, false, true>(a, *sg, num_sms, stream, info);
    return inclusive ? launch_seg_t<Op, true, false>(a, none, num_sms, stream, info)
                     : launch_seg_t<Op, false, false>(a, none, num_sms, stream, info);
}

}  // namespace gps
