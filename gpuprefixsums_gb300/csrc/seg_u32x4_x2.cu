// Generic / segmented scan, OpU32x4 (struct of four u32 members) instantiations with two threads per row.
#include "seg_launch.cuh"

namespace gps {
cudaError_t launch_seg_u32x4_x2(bool inclusive, const ScanArgs& a, const SegArgs* sg, const GenericConfig& cfg,
                              int num_sms, cudaStream_t stream, LaunchInfo* info) {
    return launch_seg_op<OpU32x4, 2>(inclusive, a, sg, cfg, num_sms, stream, info);
}
bool seg_u32x4_x2_fits(uint32_t unit) {
    if (unit == 1) return SegStages<OpU32x4, 1, true, 2>::kFits && SegStages<OpU32x4, 1, false, 2>::kFits;
    if (unit == 4) return SegStages<OpU32x4, 4, true, 2>::kFits && SegStages<OpU32x4, 4, false, 2>::kFits;
    return false;
}
}  // namespace gps
