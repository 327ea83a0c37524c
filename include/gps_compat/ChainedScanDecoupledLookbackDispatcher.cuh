/*
 * Drop-in for GPUPrefixSumsCUDA/ChainedScanDecoupledLookbackDispatcher.cuh:16-212
 * (class ChainedScanDecoupledLookbackDispatcher): same constructor and public
 * methods, backed by gps_scan(GPS_ALGO_CSDL) on the dispatcher's own buffer.
 */
#pragma once
#include "gps_compat_common.h"

class ChainedScanDecoupledLookbackDispatcher : public gps_compat::DispatcherBase {
   public:
    // ChainedScanDecoupledLookbackDispatcher.cuh:28-34
    explicit ChainedScanDecoupledLookbackDispatcher(uint32_t maxSize)
        : DispatcherBase(GPS_ALGO_CSDL, maxSize, "ChainedScanDecoupledLookback") {}

    // :38-76
    void TestAllExclusive() { TestAll(false, "exclusive"); }

    // :78-114
    void TestAllInclusive() { TestAll(true, "inclusive"); }

    // :116-156
    void BatchTimingInclusive(uint32_t size, uint32_t batchCount) {
        BatchTiming(size, batchCount, true, "GPUPrefixSums ChainedScanDecoupledLookback inclusive");
    }

    // :158-163 (the reference's main calls the destructor explicitly)
    ~ChainedScanDecoupledLookbackDispatcher() { Release(); }
};
