/*
 * Shared body of the drop-in dispatcher classes (host C++ over include/gps.h).
 *
 * The reference's dispatchers (the *Dispatcher.cuh headers of the
 * GPUPrefixSumsCUDA folder) own a u32 buffer of maxSize elements, scan it in
 * place, test themselves on all-ones input and time themselves with CUDA
 * events. These classes keep that public
 * surface -- constructor(uint32_t maxSize), TestAllExclusive(),
 * TestAllInclusive(), BatchTimingInclusive(size, batchCount), destructor --
 * and its console messages, but every scan runs through gps_scan().
 *
 * Two deliberate differences from the reference:
 *  - the large-size checks validate 2^26, 2^27 and 2^28 elements; the
 *    reference passes the exponent instead of the size to its init and
 *    validation kernels (ChainedScanDecoupledLookbackDispatcher.cuh:61-68),
 *    so it only checks the first 26-28 elements;
 *  - validation runs on the host against a serial scan (the reference counts
 *    errors with an atomic on the device, UtilityKernels.cuh:22-38).
 */
#ifndef GPS_COMPAT_COMMON_H_
#define GPS_COMPAT_COMMON_H_

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <vector>

#include "gps.h"

namespace gps_compat {

class DispatcherBase {
   protected:
    const uint32_t k_partitionSize = 4096;  // reference tile: 8 warps x 32 lanes x 4 uint4
    const uint32_t k_maxSize;
    const char* const k_name;
    uint32_t* m_scan = nullptr;
    uint32_t* m_pristine = nullptr;  // all-ones copy used to re-initialise m_scan
    gps_plan m_plan = nullptr;
    bool m_ok = false;

    static uint32_t divRoundUp(uint32_t x, uint32_t y) { return (x + y - 1) / y; }
    static uint32_t align16(uint32_t x) { return divRoundUp(x, 4) * 4; }

    DispatcherBase(gps_algo algo, uint32_t maxSize, const char* name)
        : k_maxSize(align16(maxSize)), k_name(name) {
        if (gps_plan_create(&m_plan, algo, GPS_DTYPE_U32, k_maxSize) != GPS_OK) {
            printf("%s: plan creation failed: %s\n", k_name, gps_last_error());
            return;
        }
        if (cudaMalloc(&m_scan, sizeof(uint32_t) * k_maxSize) != cudaSuccess ||
            cudaMalloc(&m_pristine, sizeof(uint32_t) * k_maxSize) != cudaSuccess) {
            printf("%s: buffer allocation failed\n", k_name);
            return;
        }
        std::vector<uint32_t> ones(k_maxSize, 1u);
        if (cudaMemcpy(m_pristine, ones.data(), sizeof(uint32_t) * k_maxSize, cudaMemcpyHostToDevice) !=
            cudaSuccess)
            return;
        m_ok = true;
    }

    virtual ~DispatcherBase() { Release(); }

    void Release() {
        if (m_scan) cudaFree(m_scan);
        if (m_pristine) cudaFree(m_pristine);
        if (m_plan) gps_plan_destroy(m_plan);
        m_scan = m_pristine = nullptr;
        m_plan = nullptr;
        m_ok = false;
    }

    // InitOne (UtilityKernels.cuh:15-20): all ones in the first `size` elements.
    void InitOne(uint32_t size) {
        cudaMemcpy(m_scan, m_pristine, sizeof(uint32_t) * size, cudaMemcpyDeviceToDevice);
    }

    bool Dispatch(uint32_t size, bool inclusive) {
        const gps_status st = gps_scan(m_plan, inclusive ? GPS_SCAN_INCLUSIVE : GPS_SCAN_EXCLUSIVE, m_scan, m_scan,
                                       size, nullptr);
        if (st != GPS_OK) {
            printf("%s: %s: %s\n", k_name, gps_status_string(st), gps_last_error());
            return false;
        }
        return true;
    }

    // ValidateInclusive / ValidateExclusive (UtilityKernels.cuh:22-38).
    bool Validate(uint32_t size, bool inclusive) {
        if (gps_plan_check(m_plan, nullptr) != GPS_OK) return false;
        std::vector<uint32_t> h(size);
        if (cudaMemcpy(h.data(), m_scan, sizeof(uint32_t) * size, cudaMemcpyDeviceToHost) != cudaSuccess)
            return false;
        for (uint32_t i = 0; i < size; ++i)
            if (h[i] != (inclusive ? i + 1 : i)) return false;
        return true;
    }

    virtual bool DispatchAndValidate(uint32_t size, bool inclusive) {
        InitOne(size);
        return Dispatch(size, inclusive) && Validate(size, inclusive);
    }

    // Tests every size in [partition, 2 * partition], then 2^26..2^28.
    void TestAll(bool inclusive, const char* testName) {
        if (k_maxSize < (1u << 28)) {
            printf("This test requires a minimum initialized size of %u. ", 1u << 28);
            printf("Reinitialize the object to at least %u.\n", 1u << 28);
            return;
        }
        if (!m_ok) {
            printf("%s: not initialised\n", k_name);
            return;
        }
        printf("Beginning GPUPrefixSums %s %s validation test: \n", k_name, testName);
        uint32_t testsPassed = 0;
        for (uint32_t i = k_partitionSize; i < k_partitionSize * 2 + 1; ++i) {
            if (DispatchAndValidate(i, inclusive))
                testsPassed++;
            else
                printf("\n Test failed at size %u \n", i);
            if (!(i & 255)) printf(".");
        }
        printf("\n");
        for (uint32_t i = 26; i <= 28; ++i) {
            if (DispatchAndValidate(1u << i, inclusive))
                testsPassed++;
            else
                printf("\n Test failed at size %u \n", 1u << i);
        }
        if (testsPassed == k_partitionSize + 3 + 1)
            printf("%u/%u All tests passed.\n\n", testsPassed, testsPassed);
        else
            printf("%u/%u Test failed.\n\n", testsPassed, k_partitionSize + 3 + 1);
    }

    // Reference timing loop (ChainedScanDecoupledLookbackDispatcher.cuh:116-156):
    // batchCount + 1 runs, the first discarded, re-initialised between runs.
    double BatchTiming(uint32_t size, uint32_t batchCount, bool inclusive, const char* title) {
        if (size > k_maxSize) {
            printf("Error, requested test size exceeds max initialized size. \n");
            return 0.0;
        }
        if (!m_ok) return 0.0;
        printf("Beginning %s batch timing test at:\n", title);
        printf("Size: %u\n", size);
        printf("Test size: %u\n", batchCount);
        cudaEvent_t start, stop;
        cudaEventCreate(&start);
        cudaEventCreate(&stop);
        float totalTime = 0.0f;
        for (uint32_t i = 0; i <= batchCount; ++i) {
            InitOne(size);
            cudaDeviceSynchronize();
            cudaEventRecord(start);
            Dispatch(size, inclusive);
            cudaEventRecord(stop);
            cudaEventSynchronize(stop);
            float millis = 0.0f;
            cudaEventElapsedTime(&millis, start, stop);
            if (i) totalTime += millis;
            if ((i & 15) == 0) printf(". ");
        }
        cudaEventDestroy(start);
        cudaEventDestroy(stop);
        printf("\n");
        totalTime /= 1000.0f;
        printf("Total time elapsed: %f\n", totalTime);
        const double keys = size / totalTime * batchCount;
        printf("Estimated speed at %u 32-bit elements: %E keys/sec\n\n", size, keys);
        return keys;
    }
};

}  // namespace gps_compat

#endif  // GPS_COMPAT_COMMON_H_
