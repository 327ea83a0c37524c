// Generic / segmented scan, OpU32x4 (struct of four u32 members) instantiations.
#include "seg_launch.cuh"

namespace gps {
cudaError_t launch_seg_u32x4(bool inclusive, const ScanArgs& a, const SegArgs* sg, const GenericConfig& cfg,
                             int num_sms, cudaStream_t stream, LaunchInfo* info) {
    return launch_seg_op<OpU32x4>(inclusive, a, sg, cfg, num_sms, stream, info);
}
}  // namespace gps
