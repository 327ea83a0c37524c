// Generic / segmented scan, OpU32 instantiations.
#include "seg_launch.cuh"

namespace gps {
cudaError_t launch_seg_u32(bool inclusive, const ScanArgs& a, const SegArgs* sg, const GenericConfig& cfg, int num_sms,
                          cudaStream_t stream, LaunchInfo* info) {
    if (cfg.split == 2) return launch_seg_u32_x2(inclusive, a, sg, cfg, num_sms, stream, info);
    return launch_seg_op<OpU32, 1>(inclusive, a, sg, cfg, num_sms, stream, info);
}
}  // namespace gps
