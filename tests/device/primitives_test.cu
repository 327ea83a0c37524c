// Kernels that exercise the device-callable primitives of include/gps_device.cuh
// for the GPU tests (built into _build/libgps_devtest.so). Each warp, block or
// tile scans its own fixed-size segment of the input; lanes past n hold the
// operator's identity.
#include <cuda_runtime.h>

#include <cstdint>

#include "gps_device.cuh"

namespace {
using namespace gps_device;

template <WarpAlgo A, typename Op>
__global__ void warp_kernel(const uint32_t* in, uint32_t* out, uint64_t n, int inclusive, int reduce) {
    const uint64_t gw = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const uint64_t i = gw * 32 + lane_id();
    const uint32_t x = i < n ? in[i] : Op::template identity<uint32_t>();
    uint32_t y;
    if (reduce)
        y = warp_reduce(x, Op());
    else if (inclusive)
        y = warp_inclusive_scan<A>(x, Op());
    else
        y = warp_exclusive_scan<A>(x, Op());
    if (i < n) out[i] = y;
}

template <int THREADS, typename Op>
__global__ void block_kernel(const uint32_t* in, uint32_t* out, uint64_t n, int inclusive, int reduce) {
    __shared__ BlockScanStorage<THREADS, uint32_t> st;
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * THREADS + threadIdx.x;
    const uint32_t x = i < n ? in[i] : Op::template identity<uint32_t>();
    uint32_t y;
    if (reduce)
        y = block_reduce<THREADS>(x, st, Op());
    else if (inclusive)
        y = block_inclusive_scan<THREADS>(x, st, Op());
    else
        y = block_exclusive_scan<THREADS>(x, st, Op());
    if (i < n) out[i] = y;
}

template <int THREADS, int ITEMS, typename Op>
__global__ void tile_kernel(const uint32_t* in, uint32_t* out, uint64_t n, int inclusive, uint32_t* totals) {
    __shared__ BlockScanStorage<THREADS, uint32_t> st;
    const uint64_t base = static_cast<uint64_t>(blockIdx.x) * THREADS * ITEMS + threadIdx.x * ITEMS;
    uint32_t v[ITEMS];
#pragma unroll
    for (int e = 0; e < ITEMS; ++e) v[e] = base + e < n ? in[base + e] : Op::template identity<uint32_t>();
    const uint32_t tot = inclusive ? tile_scan<THREADS, ITEMS, true>(v, st, Op()) : tile_scan<THREADS, ITEMS, false>(v, st, Op());
#pragma unroll
    for (int e = 0; e < ITEMS; ++e)
        if (base + e < n) out[base + e] = v[e];
    if (threadIdx.x == 0) totals[blockIdx.x] = tot;
}

template <typename Op>
int launch(int level, int algo, const uint32_t* in, uint32_t* out, uint64_t n, int inclusive, int reduce,
           uint32_t* totals) {
    if (n == 0) return 0;
    if (level == 0) {
        const unsigned blocks = static_cast<unsigned>((n + 255) / 256);
        if (algo == 0)
            warp_kernel<WarpAlgo::KoggeStone, Op><<<blocks, 256>>>(in, out, n, inclusive, reduce);
        else
            warp_kernel<WarpAlgo::Sklansky, Op><<<blocks, 256>>>(in, out, n, inclusive, reduce);
    } else if (level == 1) {
        block_kernel<256, Op><<<static_cast<unsigned>((n + 255) / 256), 256>>>(in, out, n, inclusive, reduce);
    } else if (level == 2) {
        block_kernel<1024, Op><<<static_cast<unsigned>((n + 1023) / 1024), 1024>>>(in, out, n, inclusive, reduce);
    } else {
        tile_kernel<128, 16, Op><<<static_cast<unsigned>((n + 2047) / 2048), 128>>>(in, out, n, inclusive, totals);
    }
    const cudaError_t err = cudaDeviceSynchronize();
    return err == cudaSuccess ? static_cast<int>(cudaGetLastError()) : static_cast<int>(err);
}
}  // namespace

// level: 0 warp (32), 1 block of 256, 2 block of 1024, 3 tile of 128 x 16.
// op: 0 plus, 1 max, 2 min. algo (warp level): 0 Kogge-Stone, 1 Sklansky.
extern "C" int gps_devtest_run(int level, int op, int algo, const uint32_t* in, uint32_t* out, uint64_t n,
                               int inclusive, int reduce, uint32_t* totals) {
    switch (op) {
        case 0: return launch<Plus>(level, algo, in, out, n, inclusive, reduce, totals);
        case 1: return launch<Max>(level, algo, in, out, n, inclusive, reduce, totals);
        case 2: return launch<Min>(level, algo, in, out, n, inclusive, reduce, totals);
    }
    return -1;
}

namespace {
// Holds its SM for `ns` nanoseconds of %globaltimer and exits: 1024 threads
// and 227 KB of shared memory per CTA, so no other CTA fits beside it. Used
// to run scans while part of the GPU is taken by another kernel. The wait is
// bounded by the timer alone.
__global__ void __launch_bounds__(1024, 1) occupy_kernel(unsigned long long ns) {
    extern __shared__ unsigned char held[];
    unsigned long long t0, now;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    if (threadIdx.x == 0) held[0] = 1;
    do {
        __nanosleep(2000);
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
    } while (now - t0 < ns);
}
}  // namespace

// Launches `ctas` occupying CTAs for ns nanoseconds (at most 0.2 s) on
// `stream`, without waiting for them. Returns the launch status.
extern "C" int gps_devtest_occupy(unsigned ctas, unsigned long long ns, void* stream) {
    constexpr int kSmem = 227 * 1024;
    if (ns > 200000000ull) return -1;
    cudaError_t err = cudaFuncSetAttribute(occupy_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
    if (err != cudaSuccess) return static_cast<int>(err);
    occupy_kernel<<<ctas, 1024, kSmem, static_cast<cudaStream_t>(stream)>>>(ns);
    return static_cast<int>(cudaGetLastError());
}
