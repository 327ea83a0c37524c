// Generic / segmented scan, OpF32C instantiations with two threads per row.
#include "seg_launch.cuh"

namespace gps {
cudaError_t launch_seg_f32c_x2(bool inclusive, const ScanArgs& a, const SegArgs* sg, const GenericConfig& cfg,
                              int num_sms, cudaStream_t stream, LaunchInfo* info) {
    return launch_seg_op<OpF32C, 2>(inclusive, a, sg, cfg, num_sms, stream, info);
}
bool seg_f32c_x2_fits(uint32_t unit) {
    if (unit == 1) return SegStages<OpF32C, 1, true, 2>::kFits && SegStages<OpF32C, 1, false, 2>::kFits;
    if (unit == 4) return SegStages<OpF32C, 4, true, 2>::kFits && SegStages<OpF32C, 4, false, 2>::kFits;
    return false;
}
}  // namespace gps
