// Launcher of the generic kernel (scan_seg.cuh) for one scan operation;
// included by one .cu file per operation so that the instantiations compile
// in parallel.
#pragma once
#include "launch_util.h"
#include "scan_seg.cuh"

namespace gps {

// 4 reduce + 4 finalize warps over 16 KB tiles, 6 units in flight per CTA.
// Stages: as many as fit in 227 KB of shared memory next to the control
// block (whose per-thread prefixes and head bitmaps grow with the state size
// and the unit), taken as 4 reduce-pass + 9 scan-pass stages when 13 fit
// (measured on GB300: 4 + 9 beats 5 + 8 by 3-8% on the batched workloads),
// else 4 + 8, 4 + 7, 3 + 7, 3 + 6. Four reduce-pass stages matter more than
// a scan-pass stage: with 11 stages, 4 + 7 instead of 3 + 8 took the batched
// u64 scan (3312 segments, 357 M elements) from 4.98 to 6.22 TB/s, and 3 + 8
// took batched FP32 from 6.17 down to 4.79. The unit (1 or 4 tiles) and the
// CTA count come from the plan's launch configuration (GenericConfig).
constexpr int kSegWarps = 4;
constexpr int kSegQueue = 6;
constexpr size_t kMaxSmem = 232448;

template <class Op, int G, bool SEG, int SPLIT>
struct SegStages {
    static constexpr int RW = kSegWarps * SPLIT;  // warps per role
    static constexpr bool k13 = seg_smem_bytes<Op, RW, 4, 9, kSegQueue, G, SEG>() <= kMaxSmem;
    static constexpr bool k12 = seg_smem_bytes<Op, RW, 4, 8, kSegQueue, G, SEG>() <= kMaxSmem;
    static constexpr bool k11 = seg_smem_bytes<Op, RW, 3, 8, kSegQueue, G, SEG>() <= kMaxSmem;
    static constexpr bool k10 = seg_smem_bytes<Op, RW, 3, 7, kSegQueue, G, SEG>() <= kMaxSmem;
    static constexpr int RS = (k13 || k12 || k11) ? 4 : 3;
    static constexpr int SS = k13 ? 9 : k12 ? 8 : (k11 || k10) ? 7 : 6;
    // Two threads per row double the per-thread prefixes: some types do not
    // fit 9 stages then, and that shape is not offered for them.
    static constexpr bool kFits = seg_smem_bytes<Op, RW, RS, SS, kSegQueue, G, SEG>() <= kMaxSmem;
    static_assert(kFits || SPLIT > 1, "227 KB per CTA");
};

template <class Op, bool INCL, bool SEG, int UNIT, int SPLIT>
cudaError_t launch_seg_t(const ScanArgs& a, const SegArgs& sg, const GenericConfig& cfg, int num_sms,
                         cudaStream_t stream, LaunchInfo* info) {
    using St = SegStages<Op, UNIT, SEG, SPLIT>;
    if constexpr (!St::kFits) {
        return cudaErrorNotSupported;
    } else {
    auto kern = scan_seg_kernel<Op, St::RW, St::RS, St::SS, kSegQueue, UNIT, INCL, SEG>;
    constexpr size_t smem = seg_smem_bytes<Op, St::RW, St::RS, St::SS, kSegQueue, UNIT, SEG>();
    constexpr int threads = SegShape<Op, St::RW>::kThreads;
    RowMaps maps;
    cudaError_t err = encode_row_maps(a.in, a.out, a.n, static_cast<uint32_t>(sizeof(typename Op::T)), &maps);
    if (err != cudaSuccess) return err;
    int occ = 0;
    err = resident_ctas_per_sm(kern, threads, smem, &occ);
    if (err != cudaSuccess) return err;
    const uint32_t units = (a.num_tiles + UNIT - 1) / UNIT;
    const int ctas = std::max(1, occ * num_sms / static_cast<int>(std::max(1u, cfg.ctas_div)));
    const int grid = persistent_grid(units, 1, ctas);
    if (info) *info = LaunchInfo{grid, threads, smem};
    ScanArgs b = a;
    b.desc_stride = units <= kSegStrideMaxUnits ? kSegDescStride : 0u;
    kern<<<grid, threads, smem, stream>>>(b, sg, maps.in, maps.out);
    return cudaGetLastError();
    }
}

template <class Op, int UNIT, int SPLIT>
cudaError_t launch_seg_unit(bool inclusive, const ScanArgs& a, const SegArgs* sg, const GenericConfig& cfg,
                            int num_sms, cudaStream_t stream, LaunchInfo* info) {
    const SegArgs none{nullptr, 0};
    if (sg != nullptr)
        return inclusive ? launch_seg_t<Op, true, true, UNIT, SPLIT>(a, *sg, cfg, num_sms, stream, info)
                         : launch_seg_t<Op, false, true, UNIT, SPLIT>(a, *sg, cfg, num_sms, stream, info);
    return inclusive ? launch_seg_t<Op, true, false, UNIT, SPLIT>(a, none, cfg, num_sms, stream, info)
                     : launch_seg_t<Op, false, false, UNIT, SPLIT>(a, none, cfg, num_sms, stream, info);
}

// The kernels of one scan operation and one row split (threads per row).
template <class Op, int SPLIT>
cudaError_t launch_seg_op(bool inclusive, const ScanArgs& a, const SegArgs* sg, const GenericConfig& cfg, int num_sms,
                          cudaStream_t stream, LaunchInfo* info) {
    if (cfg.split != static_cast<uint32_t>(SPLIT)) return cudaErrorInvalidValue;
    switch (cfg.unit) {
        case 1: return launch_seg_unit<Op, 1, SPLIT>(inclusive, a, sg, cfg, num_sms, stream, info);
        case 4: return launch_seg_unit<Op, 4, SPLIT>(inclusive, a, sg, cfg, num_sms, stream, info);
    }
    return cudaErrorInvalidValue;
}

}  // namespace gps
