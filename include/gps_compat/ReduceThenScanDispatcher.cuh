/*
 * Drop-in for GPUPrefixSumsCUDA/ReduceThenScanDispatcher.cuh:16-204
 * (class ReduceThenScanDispatcher): same constructor and public methods,
 * backed by gps_scan(GPS_ALGO_RTS) on the dispatcher's own buffer.
 */
#pragma once
#include "gps_compat_common.h"

class ReduceThenScanDispatcher : public gps_compat::DispatcherBase {
   public:
    // ReduceThenScanDispatcher.cuh:27-32
    explicit ReduceThenScanDispatcher(uint32_t maxSize) : DispatcherBase(GPS_ALGO_RTS, maxSize, "ReduceThenScan") {}

    // :36-73
    void TestAllExclusive() { TestAll(false, "exclusive"); }

    // :75-110
    void TestAllInclusive() { TestAll(true, "inclusive"); }

    // :112-150
    void BatchTimingInclusive(uint32_t size, uint32_t batchCount) {
        BatchTiming(size, batchCount, true, "GPUPrefixSums ReduceThenScan inclusive");
    }

    // :152-156
    ~ReduceThenScanDispatcher() { Release(); }
};
