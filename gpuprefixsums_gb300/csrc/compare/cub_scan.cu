// Comparison bar for the benchmark: CUB's DeviceScan (CCCL of the CUDA
// toolkit) compiled for sm_103a, as the reference's CubDispatcher times it
// (GPUPrefixSumsCUDA/CubDispatcher.cuh:32-76). Built as libgps_cub.so, apart
// from the scan library; nothing in libgps.so calls CUB.
#include <cub/device/device_scan.cuh>
#include <cub/device/device_select.cuh>
#include <cuda_runtime.h>

#include <cstdint>

extern "C" {

// Query (temp == nullptr) or run CUB's exclusive / inclusive sum of n u32.
int gps_cub_scan_u32(int inclusive, const void* in, void* out, uint64_t n, void* temp, size_t* temp_bytes,
                     cudaStream_t stream) {
    const uint32_t* i = static_cast<const uint32_t*>(in);
    uint32_t* o = static_cast<uint32_t*>(out);
    cudaError_t err;
    if (inclusive)
        err = cub::DeviceScan::InclusiveSum(temp, *temp_bytes, i, o, static_cast<int64_t>(n), stream);
    else
        err = cub::DeviceScan::ExclusiveSum(temp, *temp_bytes, i, o, static_cast<int64_t>(n), stream);
    return static_cast<int>(err);
}

int gps_cub_scan_u64(int inclusive, const void* in, void* out, uint64_t n, void* temp, size_t* temp_bytes,
                     cudaStream_t stream) {
    const uint64_t* i = static_cast<const uint64_t*>(in);
    uint64_t* o = static_cast<uint64_t*>(out);
    cudaError_t err;
    if (inclusive)
        err = cub::DeviceScan::InclusiveSum(temp, *temp_bytes, i, o, static_cast<int64_t>(n), stream);
    else
        err = cub::DeviceScan::ExclusiveSum(temp, *temp_bytes, i, o, static_cast<int64_t>(n), stream);
    return static_cast<int>(err);
}

// Member-wise sum of four u32 (a struct of four independent counters).
struct U32x4Plus {
    __host__ __device__ uint4 operator()(const uint4& a, const uint4& b) const {
        return make_uint4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
    }
};

// Query (temp == nullptr) or run CUB's inclusive scan of n uint4 structs with
// the member-wise sum.
int gps_cub_scan_u32x4(const void* in, void* out, uint64_t n, void* temp, size_t* temp_bytes, cudaStream_t stream) {
    return static_cast<int>(cub::DeviceScan::InclusiveScan(temp, *temp_bytes, static_cast<const uint4*>(in),
                                                           static_cast<uint4*>(out), U32x4Plus(),
                                                           static_cast<int64_t>(n), stream));
}

// Query (temp == nullptr) or run CUB's DeviceSelect::Flagged of n u32 with
// one flag byte each; the count goes to *num_selected (device, int64).
int gps_cub_select_u32(const void* in, const void* flags, void* out, void* num_selected, uint64_t n, void* temp,
                       size_t* temp_bytes, cudaStream_t stream) {
    return static_cast<int>(cub::DeviceSelect::Flagged(
        temp, *temp_bytes, static_cast<const uint32_t*>(in), static_cast<const uint8_t*>(flags),
        static_cast<uint32_t*>(out), static_cast<int64_t*>(num_selected), static_cast<int64_t>(n), stream));
}
}
