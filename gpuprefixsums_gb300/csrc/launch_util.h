// Host-side helpers for persistent launches: per-(kernel, device, context)
// cache of the dynamic shared-memory opt-in and of the occupancy that sizes
// the grid.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <map>
#include <mutex>
#include <tuple>
#include <utility>

namespace gps {

// Id of the driver context current on this thread (cuCtxGetId: unique for
// the life of the process), or 0 if there is none yet -- the runtime creates
// a device's primary context on first use. Function attributes and module
// addresses belong to a context: after cudaDeviceReset(), or in another
// driver context on the same device, they must be set up again.
inline unsigned long long current_ctx_id() {
    using GetCurrentFn = CUresult(CUDAAPI*)(CUcontext*);
    using GetIdFn = CUresult(CUDAAPI*)(CUcontext, unsigned long long*);
    static std::once_flag once;
    static GetCurrentFn get_current = nullptr;
    static GetIdFn get_id = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrentFn>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetIdFn>(p);
    });
    if (get_current == nullptr || get_id == nullptr) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Resident CTAs per SM for `kern` with `threads` threads and `smem` bytes of
// dynamic shared memory on the current device. Opts the kernel in to more
// than 48 KB of dynamic shared memory the first time it is seen on a device.
template <typename Kernel>
cudaError_t resident_ctas_per_sm(Kernel kern, int threads, size_t smem, int* out) {
    static std::mutex mu;
    static std::map<std::tuple<const void*, int, unsigned long long>, int> cache;
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return err;
    // Without a current context yet (0) nothing is cached: the calls below
    // create the primary context, and the next call finds its id.
    const unsigned long long ctx = current_ctx_id();
    const auto key = std::make_tuple(reinterpret_cast<const void*>(kern), dev, ctx);
    if (ctx != 0) {
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
    if (ctx != 0) cache[key] = occ;
    *out = occ;
    return cudaSuccess;
}

// Persistent grid: as many CTAs as can be resident, but no more than tiles.
inline int persistent_grid(uint32_t num_tiles, int ctas_per_sm, int num_sms) {
    const uint64_t cap = static_cast<uint64_t>(ctas_per_sm) * static_cast<uint64_t>(num_sms);
    return static_cast<int>(std::max<uint64_t>(1, std::min<uint64_t>(num_tiles, cap)));
}

}  // namespace gps
