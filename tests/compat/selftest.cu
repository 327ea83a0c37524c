// Exercises the drop-in dispatcher classes (include/gps_compat/) through the
// same sequence of calls the reference's driver makes
// (GPUPrefixSumsCUDA/GPUPrefixSumsCUDA.cu:14-38): construct at 2^28, run the
// exclusive and inclusive self-tests, time 2^28-element inclusive scans, and
// destroy; then the forced-stall dispatcher and the CUB comparison.
// Usage: compat_selftest [batchCount]   (default 100, as in the reference)
#include <cstdlib>

#include "ChainedScanDecoupledLookbackDispatcher.cuh"
#include "CubDispatcher.cuh"
#include "EmulatedDeadlockingDispatcher.cuh"
#include "ReduceThenScanDispatcher.cuh"

int main(int argc, char** argv) {
    const uint32_t batch = argc > 1 ? static_cast<uint32_t>(std::atoi(argv[1])) : 100u;

    ChainedScanDecoupledLookbackDispatcher* csdl = new ChainedScanDecoupledLookbackDispatcher(1 << 28);
    csdl->TestAllExclusive();
    csdl->TestAllInclusive();
    csdl->BatchTimingInclusive(1 << 28, batch);
    delete csdl;

    ReduceThenScanDispatcher* rts = new ReduceThenScanDispatcher(1 << 28);
    rts->TestAllExclusive();
    rts->TestAllInclusive();
    rts->BatchTimingInclusive(1 << 28, batch);
    delete rts;

    EmulatedDeadlockingDispatcher* ed = new EmulatedDeadlockingDispatcher(1 << 28);
    ed->TestAllInclusive();
    ed->BatchTimingInclusive(1 << 28, batch);
    delete ed;

    CubDispatcher* cub = new CubDispatcher(1 << 28);
    cub->BatchTimingCubChainedScan(1 << 28, batch);
    delete cub;
    return 0;
}
