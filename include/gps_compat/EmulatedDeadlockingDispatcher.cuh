/*
 * Drop-in for GPUPrefixSumsCUDA/EmulatedDeadlockingDispatcher.cuh:16-177
 * (class EmulatedDeadlockingDispatcher): the chained scan in forced-stall
 * mode. Every tile with (tile & partMask) == 0 withholds its aggregate until a
 * successor whose lookback made no progress for maxSpinCount polls re-reduces
 * the tile's input and inserts it (EmulatedDeadlocking.cuh:64-150). Unlike the
 * reference, whose kernel ignores these two arguments (compile-time
 * MAX_SPIN_COUNT 4 / DEADLOCK_MASK 7, EmulatedDeadlocking.cuh:15-16), the
 * values passed are used, and every wait is bounded.
 */
#pragma once
#include <fstream>

#include "gps_compat_common.h"

class EmulatedDeadlockingDispatcher : public gps_compat::DispatcherBase {
    // A stalled tile with no successor (the last tile) is released after this
    // delay; the reference would wait for ever there.
    static constexpr uint32_t kStallDelayNs = 20u * 1000u * 1000u;

    void Configure(uint32_t partMask, uint32_t maxSpinCount) {
        gps_plan_set_stall(m_plan, 1, partMask + 1, 0, kStallDelayNs, maxSpinCount ? maxSpinCount : 1);
    }

   public:
    // EmulatedDeadlockingDispatcher.cuh:29-36
    explicit EmulatedDeadlockingDispatcher(uint32_t maxSize)
        : DispatcherBase(GPS_ALGO_CSDL, maxSize, "EmulatedDeadlocking") {
        if (m_ok) Configure(7, 4);
    }

    // :41-77
    void TestAllInclusive() {
        Configure(7, 4);
        TestAll(true, "inclusive");
    }

    // :79-126
    double BatchTimingInclusive(uint32_t size, uint32_t batchCount, uint32_t partMask, uint32_t maxSpinCount) {
        Configure(partMask, maxSpinCount);
        const double keys = BatchTiming(size, batchCount, true, "Emulated Deadlocking");
        Configure(7, 4);
        return keys;
    }

    // :123-126
    void BatchTimingInclusive(uint32_t size, uint32_t batchCount) { BatchTimingInclusive(size, batchCount, 1, 8); }

    // :128-138
    void RecordTimingData(uint32_t spinCount) {
        std::ofstream writer;
        writer.open("data.txt");
        writer << "Max Spin Count: " << spinCount << "\n";
        for (uint32_t i = 512; i >= 64; i >>= 1) {
            const double t = BatchTimingInclusive(1u << 28, 250, i - 1, spinCount);
            writer << t << "\n";
        }
        writer.close();
    }

    // :140-145
    ~EmulatedDeadlockingDispatcher() { Release(); }
};
