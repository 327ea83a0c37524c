// Host-side helpers for persistent launches: per-(kernel, device) cache of the
// dynamic shared-memory opt-in and of the occupancy that sizes the grid.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <map>
#include <mutex>
#include <utility>

namespace gps {

// Resident CTAs per SM for `kern` with `threads` threads and `smem` bytes of
// dynamic shared memory on the current device. Opts the kernel in to more
// than 48 KB of dynamic shared memory the first time it is seen on a device.
template <typename Kernel>
cudaError_t resident_ctas_per_sm(Kernel kern, int threads, size_t smem, int* out) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, int> cache;
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return err;
    const auto key = std::make_pair(reinterpret_cast<const void*>(kern), dev);
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = cache.find(key);
        if (it != cache.end()) {
            *out = it->second;
            return cudaSuccess;
        }
    }
    if (smem > 48 * 1024) {
        err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (err != cudaSuccess) return err;
    }
    int occ = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, smem);
    if (err != cudaSuccess) return err;
    occ = std::max(occ, 1);
    std::lock_guard<std::mutex> lock(mu);
    cache[key] = occ;
    *out = occ;
    return cudaSuccess;
}

// Persistent grid: as many CTAs as can be resident, but no more than tiles.
inline int persistent_grid(uint32_t num_tiles, int ctas_per_sm, int num_sms) {
    const uint64_t cap = static_cast<uint64_t>(ctas_per_sm) * static_cast<uint64_t>(num_sms);
    return static_cast<int>(std::max<uint64_t>(1, std::min<uint64_t>(num_tiles, cap)));
}

}  // namespace gps
