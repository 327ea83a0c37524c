// Launcher of the generic kernel (scan_seg.cuh) for one scan operation;
// included by one .cu file per operation so that the instantiations compile
// in parallel.
#pragma once
#include "launch_util.h"
#include "scan_seg.cuh"

namespace gps {

// 4 reduce + 4 finalize warps over 16 KB tiles, 4 reduce-pass and 9
// scan-pass stages, 6 units in flight per CTA (measured on GB300: 4 + 9
// beats 5 + 8 by 3-8% on the batched workloads). The unit (1 or 4 tiles) and
// the CTA count come from the plan's launch configuration (GenericConfig).
constexpr int kSegWarps = 4;
constexpr int kSegRStages = 4;
constexpr int kSegSStages = 9;
constexpr int kSegQueue = 6;

template <class Op, bool INCL, bool SEG, int UNIT>
cudaError_t launch_seg_t(const ScanArgs& a, const SegArgs& sg, const GenericConfig& cfg, int num_sms,
                         cudaStream_t stream, LaunchInfo* info) {
    auto kern = scan_seg_kernel<Op, kSegWarps, kSegRStages, kSegSStages, kSegQueue, UNIT, INCL, SEG>;
    constexpr size_t smem = seg_smem_bytes<Op, kSegWarps, kSegRStages, kSegSStages, kSegQueue, UNIT, SEG>();
    static_assert(smem <= 232448, "227 KB of shared memory per CTA");
    constexpr int threads = SegShape<Op, kSegWarps>::kThreads;
    int occ = 0;
    cudaError_t err = resident_ctas_per_sm(kern, threads, smem, &occ);
    if (err != cudaSuccess) return err;
    const uint32_t units = (a.num_tiles + UNIT - 1) / UNIT;
    const int ctas = std::max(1, occ * num_sms / static_cast<int>(std::max(1u, cfg.ctas_div)));
    const int grid = persistent_grid(units, 1, ctas);
    if (info) *info = LaunchInfo{grid, threads, smem};
    kern<<<grid, threads, smem, stream>>>(a, sg);
    return cudaGetLastError();
}

template <class Op, int UNIT>
cudaError_t launch_seg_unit(bool inclusive, const ScanArgs& a, const SegArgs* sg, const GenericConfig& cfg,
                            int num_sms, cudaStream_t stream, LaunchInfo* info) {
    const SegArgs none{nullptr, 0};
    if (sg != nullptr)
        return inclusive ? launch_seg_t<Op, true, true, UNIT>(a, *sg, cfg, num_sms, stream, info)
                         : launch_seg_t<Op, false, true, UNIT>(a, *sg, cfg, num_sms, stream, info);
    return inclusive ? launch_seg_t<Op, true, false, UNIT>(a, none, cfg, num_sms, stream, info)
                     : launch_seg_t<Op, false, false, UNIT>(a, none, cfg, num_sms, stream, info);
}

template <class Op>
cudaError_t launch_seg_op(bool inclusive, const ScanArgs& a, const SegArgs* sg, const GenericConfig& cfg, int num_sms,
                          cudaStream_t stream, LaunchInfo* info) {
    switch (cfg.unit) {
        case 1: return launch_seg_unit<Op, 1>(inclusive, a, sg, cfg, num_sms, stream, info);
        case 4: return launch_seg_unit<Op, 4>(inclusive, a, sg, cfg, num_sms, stream, info);
    }
    return cudaErrorInvalidValue;
}

}  // namespace gps
