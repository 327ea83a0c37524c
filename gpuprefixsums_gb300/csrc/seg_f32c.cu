// Generic / segmented scan, OpF32C instantiations.
#include "seg_launch.cuh"

namespace gps {
cudaError_t launch_seg_f32c(bool inclusive, const ScanArgs& a, const SegArgs* sg, const GenericConfig& cfg, int num_sms,
                          cudaStream_t stream, LaunchInfo* info) {
    if (cfg.split == 2) return launch_seg_f32c_x2(inclusive, a, sg, cfg, num_sms, stream, info);
    return launch_seg_op<OpF32C, 1>(inclusive, a, sg, cfg, num_sms, stream, info);
}
}  // namespace gps
