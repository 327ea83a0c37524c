// Reference kernels for parity tests -- TEST INFRASTRUCTURE ONLY.
//
// Compiled by oracle/build.py with the reference's GPUPrefixSumsCUDA folder on
// the include path, into a device-only cubin under oracle/_ref/. Nothing here
// re-implements the reference: the headers are included unmodified and their
// kernel templates are instantiated with the reference's own tuning
// (CSDL_WARPS / RTS_WARPS = 8, UINT4_PER_THREAD = 4,
// ChainedScanDecoupledLookbackDispatcher.cuh:13-14, ReduceThenScanDispatcher.cuh:13-14;
// SpineScan<32, 4> launched <<<1, 1024>>>, ReduceThenScanDispatcher.cuh:168).
// The tests look the kernels up by name in the loaded module and launch them
// exactly as the reference dispatchers do.
#include "ChainedScanDecoupledLookback.cuh"
#include "ReduceThenScan.cuh"
#include "UtilityKernels.cuh"

template __global__ void ChainedScanDecoupledLookback::CSDLExclusive<8, 4>(uint32_t*, volatile uint32_t*,
                                                                          volatile uint32_t*, const uint32_t);
template __global__ void ChainedScanDecoupledLookback::CSDLInclusive<8, 4>(uint32_t*, volatile uint32_t*,
                                                                          volatile uint32_t*, const uint32_t);
template __global__ void ReduceThenScan::Reduce<8, 4>(uint32_t*, uint32_t*, const uint32_t);
template __global__ void ReduceThenScan::SpineScan<32, 4>(uint32_t*, const uint32_t);
template __global__ void ReduceThenScan::PropagateInclusive<8, 4>(uint32_t*, uint32_t*, const uint32_t);
template __global__ void ReduceThenScan::PropagateExclusive<8, 4>(uint32_t*, uint32_t*, const uint32_t);

