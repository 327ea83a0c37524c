/*
 * Drop-in for GPUPrefixSumsCUDA/CubDispatcher.cuh:21-77 (class CubDispatcher):
 * the reference's comparison bar, CUB's DeviceScan::InclusiveSum on the same
 * buffer, timed the same way. Needs nvcc (it instantiates CUB kernels); it is
 * a comparison tool, not part of the scan library.
 */
#pragma once
#include <cub/device/device_scan.cuh>

#include "gps_compat_common.h"

class CubDispatcher {
    const uint32_t k_maxSize;
    uint32_t* m_scan = nullptr;
    uint32_t* m_pristine = nullptr;

   public:
    explicit CubDispatcher(uint32_t size) : k_maxSize(size) {
        cudaMalloc(&m_scan, sizeof(uint32_t) * k_maxSize);
        cudaMalloc(&m_pristine, sizeof(uint32_t) * k_maxSize);
        std::vector<uint32_t> ones(k_maxSize, 1u);
        cudaMemcpy(m_pristine, ones.data(), sizeof(uint32_t) * k_maxSize, cudaMemcpyHostToDevice);
    }

    ~CubDispatcher() {
        if (m_scan) cudaFree(m_scan);
        if (m_pristine) cudaFree(m_pristine);
        m_scan = m_pristine = nullptr;
    }

    void BatchTimingCubChainedScan(uint32_t size, uint32_t batchCount) {
        if (size > k_maxSize) {
            printf("Error, requested test size exceeds max initialized size. \n");
            return;
        }
        printf("Beginning CUB ChainedScanDecoupledLookback inclusive batch timing test at:\n");
        printf("Size: %u\n", size);
        printf("Test size: %u\n", batchCount);
        void* d_temp_storage = nullptr;
        size_t temp_storage_bytes = 0;
        cub::DeviceScan::InclusiveSum(d_temp_storage, temp_storage_bytes, m_scan, size);
        cudaMalloc(&d_temp_storage, temp_storage_bytes);
        cudaEvent_t start, stop;
        cudaEventCreate(&start);
        cudaEventCreate(&stop);
        float totalTime = 0.0f;
        for (uint32_t i = 0; i <= batchCount; ++i) {
            cudaMemcpy(m_scan, m_pristine, sizeof(uint32_t) * size, cudaMemcpyDeviceToDevice);
            cudaDeviceSynchronize();
            cudaEventRecord(start);
            cub::DeviceScan::InclusiveSum(d_temp_storage, temp_storage_bytes, m_scan, size);
            cudaEventRecord(stop);
            cudaEventSynchronize(stop);
            float millis = 0.0f;
            cudaEventElapsedTime(&millis, start, stop);
            if (i) totalTime += millis;
            if ((i & 15) == 0) printf(". ");
        }
        cudaEventDestroy(start);
        cudaEventDestroy(stop);
        cudaFree(d_temp_storage);
        printf("\n");
        totalTime /= 1000.0f;
        printf("Total time elapsed: %f\n", totalTime);
        printf("Estimated speed at %u 32-bit elements: %E keys/sec\n\n", size, size / totalTime * batchCount);
    }
};
