/*
 * gps_device.cuh -- device-callable scan primitives (header only, sm_103a).
 *
 * The warp-, block- and thread-level building blocks the library's kernels
 * are made of, for use inside other kernels (radix-sort digit counts,
 * compaction inside a block, ...). Any associative operator with an identity
 * works; `Plus`, `Max` and `Min` are provided.
 *
 * The reference surveys the classic variants of these primitives in its
 * D3D12 harness (GPUPrefixSumsD3D12/Shaders/Survey.hlsl:49-1078: serial,
 * Kogge-Stone, Sklansky, Brent-Kung, raking, reduce-then-scan) and uses a
 * shuffle Kogge-Stone warp scan in its CUDA kernels (Utils.cuh:22-71). Here:
 *   warp    Kogge-Stone (shfl.up, log2(32) dependent steps, every lane
 *           busy) and Sklansky (each step broadcasts the last lane of the
 *           lower half of every 2d-lane group);
 *   block   raking over warp totals: each warp scans, the warp totals go
 *           through shared memory and every warp scans them again;
 *           THREADS a multiple of 32, at most 1024;
 *   thread  serial scan of ITEMS values in registers, and the "items per
 *           thread" tile scan that composes the three.
 * All functions must be called by every thread of the warp (block) with
 * the full mask active.
 */
#ifndef GPS_DEVICE_CUH_
#define GPS_DEVICE_CUH_

#include <cuda_runtime.h>
#include <stdint.h>

namespace gps_device {

struct Plus {
    template <typename T>
    __device__ __forceinline__ T operator()(T a, T b) const { return a + b; }
    template <typename T>
    __device__ __forceinline__ static T identity() { return T(0); }
};

struct Max {
    template <typename T>
    __device__ __forceinline__ T operator()(T a, T b) const { return a > b ? a : b; }
    template <typename T>
    __device__ __forceinline__ static T identity();
};
template <>
__device__ __forceinline__ uint32_t Max::identity<uint32_t>() { return 0u; }
template <>
__device__ __forceinline__ uint64_t Max::identity<uint64_t>() { return 0ull; }
template <>
__device__ __forceinline__ int32_t Max::identity<int32_t>() { return INT32_MIN; }
template <>
__device__ __forceinline__ float Max::identity<float>() { return -__int_as_float(0x7f800000); }

struct Min {
    template <typename T>
    __device__ __forceinline__ T operator()(T a, T b) const { return a < b ? a : b; }
    template <typename T>
    __device__ __forceinline__ static T identity();
};
template <>
__device__ __forceinline__ uint32_t Min::identity<uint32_t>() { return 0xFFFFFFFFu; }
template <>
__device__ __forceinline__ uint64_t Min::identity<uint64_t>() { return ~0ull; }
template <>
__device__ __forceinline__ int32_t Min::identity<int32_t>() { return INT32_MAX; }
template <>
__device__ __forceinline__ float Min::identity<float>() { return __int_as_float(0x7f800000); }

enum class WarpAlgo { KoggeStone, Sklansky };

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// ------------------------------------------------------------------- warp
template <WarpAlgo A = WarpAlgo::KoggeStone, typename T, typename Op = Plus>
__device__ __forceinline__ T warp_inclusive_scan(T x, Op op = Op()) {
    const uint32_t lane = lane_id();
    if (A == WarpAlgo::KoggeStone) {
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const T y = __shfl_up_sync(0xFFFFFFFFu, x, d);
            if (lane >= static_cast<uint32_t>(d)) x = op(y, x);
        }
    } else {
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            // Lanes in the upper half of each 2d-lane group take the last
            // lane of the lower half.
            const T y = __shfl_sync(0xFFFFFFFFu, x, (lane & ~static_cast<uint32_t>(2 * d - 1)) + d - 1);
            if (lane & static_cast<uint32_t>(d)) x = op(y, x);
        }
    }
    return x;
}

// Exclusive scan; lane 0 gets the identity. The warp total is returned in
// *total when total is not null.
template <WarpAlgo A = WarpAlgo::KoggeStone, typename T, typename Op = Plus>
__device__ __forceinline__ T warp_exclusive_scan(T x, Op op = Op(), T* total = nullptr) {
    const T inc = warp_inclusive_scan<A>(x, op);
    const T exc = __shfl_up_sync(0xFFFFFFFFu, inc, 1);
    if (total) *total = __shfl_sync(0xFFFFFFFFu, inc, 31);
    return lane_id() == 0 ? Op::template identity<T>() : exc;
}

// Reduction; every lane gets the result (butterfly).
template <typename T, typename Op = Plus>
__device__ __forceinline__ T warp_reduce(T x, Op op = Op()) {
#pragma unroll
    for (int m = 16; m; m >>= 1) x = op(x, __shfl_xor_sync(0xFFFFFFFFu, x, m));
    return x;
}

// ------------------------------------------------------------------ block
// Shared memory a block scan of THREADS threads needs: one T per warp.
template <int THREADS, typename T>
struct BlockScanStorage {
    static_assert(THREADS % 32 == 0 && THREADS <= 1024, "THREADS: a multiple of 32, at most 1024");
    T warp_totals[THREADS / 32];
};

// Block scans: each warp scans its 32 values, the warp totals go through
// shared memory, and every warp scans the (at most 32) warp totals itself --
// one shared load per lane and one more warp scan instead of a second round
// of barriers. *block_total (if not null) receives the block's total in
// every thread. Contain __syncthreads().
template <int THREADS, typename T, typename Op>
__device__ __forceinline__ void block_prefix_of_warp(const BlockScanStorage<THREADS, T>& st, Op op, T& pre, T& tot) {
    constexpr int W = THREADS / 32;
    const uint32_t lane = lane_id();
    const uint32_t warp = threadIdx.x >> 5;
    T t = lane < static_cast<uint32_t>(W) ? st.warp_totals[lane] : Op::template identity<T>();
    t = warp_inclusive_scan<WarpAlgo::KoggeStone>(t, op);
    const T before = __shfl_sync(0xFFFFFFFFu, t, warp == 0 ? 0u : warp - 1);
    pre = warp == 0 ? Op::template identity<T>() : before;
    tot = __shfl_sync(0xFFFFFFFFu, t, W - 1);
}

template <int THREADS, typename T, typename Op = Plus>
__device__ __forceinline__ T block_inclusive_scan(T x, BlockScanStorage<THREADS, T>& st, Op op = Op(),
                                                  T* block_total = nullptr) {
    const uint32_t lane = lane_id();
    const uint32_t warp = threadIdx.x >> 5;
    const T inc = warp_inclusive_scan<WarpAlgo::KoggeStone>(x, op);
    if (lane == 31) st.warp_totals[warp] = inc;
    __syncthreads();
    T pre, tot;
    block_prefix_of_warp(st, op, pre, tot);
    if (block_total) *block_total = tot;
    __syncthreads();  // the storage may be reused right after
    return op(pre, inc);
}

template <int THREADS, typename T, typename Op = Plus>
__device__ __forceinline__ T block_exclusive_scan(T x, BlockScanStorage<THREADS, T>& st, Op op = Op(),
                                                  T* block_total = nullptr) {
    const uint32_t lane = lane_id();
    const uint32_t warp = threadIdx.x >> 5;
    T wt;
    const T exc = warp_exclusive_scan<WarpAlgo::KoggeStone>(x, op, &wt);
    if (lane == 0) st.warp_totals[warp] = wt;
    __syncthreads();
    T pre, tot;
    block_prefix_of_warp(st, op, pre, tot);
    if (block_total) *block_total = tot;
    __syncthreads();
    return op(pre, exc);
}

template <int THREADS, typename T, typename Op = Plus>
__device__ __forceinline__ T block_reduce(T x, BlockScanStorage<THREADS, T>& st, Op op = Op()) {
    constexpr int W = THREADS / 32;
    const uint32_t lane = lane_id();
    const uint32_t warp = threadIdx.x >> 5;
    const T w = warp_reduce(x, op);
    if (lane == 0) st.warp_totals[warp] = w;
    __syncthreads();
    T t = lane < static_cast<uint32_t>(W) ? st.warp_totals[lane] : Op::template identity<T>();
    t = warp_reduce(t, op);
    __syncthreads();
    return t;
}

// ----------------------------------------------------------------- thread
// Serial inclusive scan of ITEMS register values starting from `carry`;
// returns the total (carry included).
template <int ITEMS, typename T, typename Op = Plus>
__device__ __forceinline__ T thread_inclusive_scan(T (&v)[ITEMS], T carry, Op op = Op()) {
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
        carry = op(carry, v[i]);
        v[i] = carry;
    }
    return carry;
}

template <int ITEMS, typename T, typename Op = Plus>
__device__ __forceinline__ T thread_exclusive_scan(T (&v)[ITEMS], T carry, Op op = Op()) {
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
        const T x = v[i];
        v[i] = carry;
        carry = op(carry, x);
    }
    return carry;
}

// Tile scan: each of THREADS threads holds ITEMS consecutive values of a
// THREADS * ITEMS tile (thread t holds [t * ITEMS, (t + 1) * ITEMS)). Scans
// the tile in place (inclusive or exclusive) and returns the tile total.
template <int THREADS, int ITEMS, bool INCLUSIVE, typename T, typename Op = Plus>
__device__ __forceinline__ T tile_scan(T (&v)[ITEMS], BlockScanStorage<THREADS, T>& st, Op op = Op()) {
    T agg = Op::template identity<T>();
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) agg = op(agg, v[i]);
    T total;
    const T before = block_exclusive_scan<THREADS>(agg, st, op, &total);
    if (INCLUSIVE)
        thread_inclusive_scan(v, before, op);
    else
        thread_exclusive_scan(v, before, op);
    return total;
}

}  // namespace gps_device

#endif  // GPS_DEVICE_CUH_
