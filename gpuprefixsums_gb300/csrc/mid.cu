// Single-pass chained scan for mid-size inputs: one 16 KB tile per CTA.
//
// The persistent L2-buffered kernel (scan_l2.cuh) pays a pipeline latency of
// about 10 us per launch (unit claim, HBM load, reduce, lookback, reload from
// L2, scan, store), which dominates at small sizes. Here every tile
// gets its own CTA of 256 threads and stays in registers between the two
// halves of the scan, as in the reference's single-pass kernel
// (ChainedScanDecoupledLookback.cuh:79-139):
//   1. take a tile id: the block index when the whole grid is resident at
//      once (every CTA it may wait on is running), else from the plan's
//      atomic counter (ids follow the order in which CTAs start, so a CTA
//      only waits on CTAs already running);
//   2. load the tile (one bulk copy into shared memory for 16-byte-aligned
//      buffers, else element by element); each thread sums its 64
//      consecutive bytes (16 u32 or 8 u64) and the thread sums are
//      block-scanned (include/gps_device.cuh);
//   3. publish the tile aggregate, and let warp 0 walk back over the
//      predecessors' descriptors (the same 8- or 16-byte descriptors, epoch
//      and lookback as the L2 kernel: lookback() in scan_pipeline.cuh, here
//      re-polling without back-off for the first polls: the predecessors'
//      descriptors are typically microseconds away, not a unit's pipeline);
//   4. publish the inclusive prefix, add the prefix, store.
// The last CTA to be done with the descriptors resets the counters and
// advances the epoch, as the L2 kernel does, so the two kernels share a
// plan's scratch.
#include "gps_device.cuh"
#include "gps_internal.h"
#include "launch_util.h"
#include "scan_pipeline.cuh"

namespace gps {
namespace {

constexpr int kMidThreads = 256;

// The last CTA to be done with the descriptors (its lookback finished and its
// inclusive prefix published) returns the counters to zero and advances the
// epoch, which retires every descriptor of this launch. Called by one thread
// per CTA once its descriptor traffic is over; the output stores need no
// ordering against it, so it runs while they drain.
template <typename T>
__device__ __forceinline__ void retire_launch(const ScanArgs& a, uint32_t epoch, bool block_ids) {
    using D = DescTraits<T>;
    __threadfence();
    const uint32_t prev = atomicAdd(&a.hdr->exit_counter, 1u);
    if (prev == gridDim.x - 1) {
        __threadfence();
        if (!block_ids) a.hdr->tile_counter = 0;
        a.hdr->exit_counter = 0;
        uint32_t e = epoch + 1;
        if ((e & kEpochMask) == 0) {
            typename D::word* desc = static_cast<typename D::word*>(a.desc);
            for (unsigned long long q = 0; q < a.hdr->capacity_tiles; ++q) D::store(desc + q, D::zero());
            e += 1;
        }
        __threadfence();
        a.hdr->epoch = e;
    }
}

// Buffers not aligned to 16 bytes: each thread loads and stores its 64
// bytes element by element.
template <typename T, bool INCL>
__global__ void __launch_bounds__(kMidThreads, 2) mid_scan_kernel(const ScanArgs a, bool block_ids) {
    constexpr int TILE = 16384 / static_cast<int>(sizeof(T));
    constexpr int ITEMS = TILE / kMidThreads;  // 16 u32 or 8 u64: 64 bytes
    using D = DescTraits<T>;
    using word = typename D::word;
    __shared__ gps_device::BlockScanStorage<kMidThreads, T> st;
    __shared__ uint32_t s_tile;
    __shared__ T s_prefix;

    const uint32_t tid = threadIdx.x;
    const uint32_t lane = tid & 31u;
    if (!block_ids) {
        if (tid == 0) s_tile = atomicAdd(&a.hdr->tile_counter, 1u);
        __syncthreads();
    }
    const uint32_t t = block_ids ? blockIdx.x : s_tile;
    const uint32_t epoch = ld_volatile_u32(&a.hdr->epoch);
    const T* in = static_cast<const T*>(a.in);
    T* out = static_cast<T*>(a.out);
    const uint64_t i0 = static_cast<uint64_t>(t) * TILE + static_cast<uint64_t>(tid) * ITEMS;

    T v[ITEMS];
#pragma unroll
    for (int e = 0; e < ITEMS; ++e) v[e] = i0 + e < a.n ? in[i0 + e] : T(0);
    T sum = 0;
#pragma unroll
    for (int e = 0; e < ITEMS; ++e) sum += v[e];
    T total;
    const T before = gps_device::block_exclusive_scan<kMidThreads>(sum, st, gps_device::Plus(), &total);

    word* desc = static_cast<word*>(a.desc);
    const T carry = a.carry_in != nullptr ? *static_cast<const T*>(a.carry_in) : T(0);
    if (tid < 32) {
        if (lane == 0)
            D::store(desc + t, t == 0 ? D::pack(kInclusive, epoch, carry + total) : D::pack(kAggregate, epoch, total));
        const T pre = t == 0 ? carry : lookback<T, TILE, false, 64>(a, t, epoch, lane, carry, -1, T(0));
        if (lane == 0) {
            if (t != 0) D::store(desc + t, D::pack(kInclusive, epoch, pre + total));
            if (a.carry_out != nullptr && t == a.num_tiles - 1) *static_cast<T*>(a.carry_out) = pre + total;
            s_prefix = pre;
        }
    }
    __syncthreads();

    T run = s_prefix + before;
#pragma unroll
    for (int e = 0; e < ITEMS; ++e) {
        const T x = v[e];
        if (INCL) {
            run += x;
            v[e] = run;
        } else {
            v[e] = run;
            run += x;
        }
    }
#pragma unroll
    for (int e = 0; e < ITEMS; ++e)
        if (i0 + e < a.n) out[i0 + e] = v[e];
    if (tid == 0) retire_launch<T>(a, epoch, block_ids);
}

// The same scan for 16-byte-aligned buffers, with the tile moved by one bulk
// copy each way (cp.async.bulk into and out of shared memory) instead of
// strided per-thread accesses. Each thread reads its four 16-byte chunks in
// an order rotated by (tid >> 1) & 3, which spreads every quarter-warp over
// all 32 banks; rotated_chunk_prefix() undoes the rotation arithmetically.
template <typename T, bool INCL>
__global__ void __launch_bounds__(kMidThreads, 2) mid_bulk_kernel(const ScanArgs a, bool block_ids) {
    constexpr int TILE = 16384 / static_cast<int>(sizeof(T));
    constexpr int ITEMS = TILE / kMidThreads;
    constexpr int EPC = 16 / static_cast<int>(sizeof(T));
    constexpr int CHUNKS = ITEMS / EPC;  // 4
    using D = DescTraits<T>;
    using word = typename D::word;
    __shared__ __align__(128) T tile[TILE];
    __shared__ uint64_t bar;
    __shared__ gps_device::BlockScanStorage<kMidThreads, T> st;
    __shared__ uint32_t s_tile;
    __shared__ T s_prefix;

    const uint32_t tid = threadIdx.x;
    const uint32_t lane = tid & 31u;
    if (tid == 0) {
        if (!block_ids) s_tile = atomicAdd(&a.hdr->tile_counter, 1u);
        ptx::mbar_init(&bar, 1);
        ptx::fence_mbar_init();
    }
    __syncthreads();
    const uint32_t t = block_ids ? blockIdx.x : s_tile;
    const uint32_t epoch = ld_volatile_u32(&a.hdr->epoch);
    const uint64_t t0 = static_cast<uint64_t>(t) * TILE;
    const uint32_t cnt = static_cast<uint32_t>(min(static_cast<uint64_t>(TILE), a.n - t0));
    const uint32_t bulk = (cnt * static_cast<uint32_t>(sizeof(T))) & ~15u;
    const uint32_t bulk_elems = bulk / static_cast<uint32_t>(sizeof(T));
    const T* in = static_cast<const T*>(a.in);
    T* out = static_cast<T*>(a.out);
    if (tid == 0) {
        ptx::mbar_arrive_expect_tx(&bar, bulk);
        if (bulk) ptx::bulk_load(tile, in + t0, bulk, &bar);
    }
    // The ragged end of the last tile (under 16 bytes) by plain loads.
    if (tid < cnt - bulk_elems) tile[bulk_elems + tid] = in[t0 + bulk_elems + tid];
    const bool landed =
        ptx::mbar_try_wait(&bar, 0) || ptx::mbar_wait_bounded(&bar, 0, ptx::global_timer_ns() + a.wait_budget_ns);
    if (!landed) raise_error(a.hdr, kErrPipelineTimeout);
    __syncthreads();

    const uint32_t rot = (tid >> 1) & (CHUNKS - 1);
    const bool whole = (tid + 1) * ITEMS <= cnt;
    T v[ITEMS];
    T cs[CHUNKS];
#pragma unroll
    for (int c8 = 0; c8 < CHUNKS; ++c8) {
        const uint32_t c = (c8 + rot) & (CHUNKS - 1);
        const Chunk<T> q = *reinterpret_cast<const Chunk<T>*>(tile + tid * ITEMS + c * EPC);
        T x = 0;
#pragma unroll
        for (int e = 0; e < EPC; ++e) {
            const T y = (whole || tid * ITEMS + c * EPC + e < cnt) ? q.v[e] : T(0);
            v[c8 * EPC + e] = y;
            x += y;
        }
        cs[c8] = x;
    }
    T cpre[CHUNKS];
    T sum;
    rotated_chunk_prefix<T, CHUNKS>(cs, rot, cpre, sum);
    T total;
    const T before = gps_device::block_exclusive_scan<kMidThreads>(sum, st, gps_device::Plus(), &total);

    word* desc = static_cast<word*>(a.desc);
    const T carry = a.carry_in != nullptr ? *static_cast<const T*>(a.carry_in) : T(0);
    if (tid < 32) {
        if (lane == 0)
            D::store(desc + t, t == 0 ? D::pack(kInclusive, epoch, carry + total) : D::pack(kAggregate, epoch, total));
        const T pre = t == 0 ? carry : lookback<T, TILE, false, 64>(a, t, epoch, lane, carry, -1, T(0));
        if (lane == 0) {
            if (t != 0) D::store(desc + t, D::pack(kInclusive, epoch, pre + total));
            if (a.carry_out != nullptr && t == a.num_tiles - 1) *static_cast<T*>(a.carry_out) = pre + total;
            s_prefix = pre;
        }
    }
    __syncthreads();

    const T base = s_prefix + before;
#pragma unroll
    for (int c8 = 0; c8 < CHUNKS; ++c8) {
        T acc = base + cpre[c8];
        Chunk<T> q;
#pragma unroll
        for (int e = 0; e < EPC; ++e) {
            const T x = v[c8 * EPC + e];
            if (INCL) {
                acc += x;
                q.v[e] = acc;
            } else {
                q.v[e] = acc;
                acc += x;
            }
        }
        const uint32_t c = (c8 + rot) & (CHUNKS - 1);
        *reinterpret_cast<Chunk<T>*>(tile + tid * ITEMS + c * EPC) = q;
    }
    ptx::fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0 && bulk) {
        ptx::bulk_store(out + t0, tile, bulk);
        ptx::bulk_commit();
    }
    if (tid < cnt - bulk_elems) out[t0 + bulk_elems + tid] = tile[bulk_elems + tid];
    if (tid == 0) {
        retire_launch<T>(a, epoch, block_ids);
        // The store must have read the tile before the CTA's shared memory
        // goes away.
        if (bulk) ptx::bulk_wait_read<0>();
    }
}

template <typename T, bool INCL, bool VEC>
cudaError_t launch_mid_v(const ScanArgs& a, int num_sms, cudaStream_t stream, LaunchInfo* info) {
    auto kern = VEC ? mid_bulk_kernel<T, INCL> : mid_scan_kernel<T, INCL>;
    int occ = 0;
    cudaError_t err = resident_ctas_per_sm(kern, kMidThreads, 0, &occ);
    if (err != cudaSuccess) return err;
    const int grid = static_cast<int>(a.num_tiles);
    const bool block_ids = static_cast<int64_t>(grid) <= static_cast<int64_t>(occ) * num_sms;
    if (info) *info = LaunchInfo{grid, kMidThreads, 0};
    kern<<<grid, kMidThreads, 0, stream>>>(a, block_ids);
    return cudaGetLastError();
}

template <typename T, bool INCL>
cudaError_t launch_mid_t(const ScanArgs& a, int num_sms, cudaStream_t stream, LaunchInfo* info) {
    const bool vec = ((reinterpret_cast<uintptr_t>(a.in) | reinterpret_cast<uintptr_t>(a.out)) & 15u) == 0;
    return vec ? launch_mid_v<T, INCL, true>(a, num_sms, stream, info)
               : launch_mid_v<T, INCL, false>(a, num_sms, stream, info);
}

}  // namespace

cudaError_t launch_mid(gps_dtype dtype, bool inclusive, const ScanArgs& a, int num_sms, cudaStream_t stream,
                       LaunchInfo* info) {
    if (dtype == GPS_DTYPE_U64)
        return inclusive ? launch_mid_t<uint64_t, true>(a, num_sms, stream, info)
                         : launch_mid_t<uint64_t, false>(a, num_sms, stream, info);
    return inclusive ? launch_mid_t<uint32_t, true>(a, num_sms, stream, info)
                     : launch_mid_t<uint32_t, false>(a, num_sms, stream, info);
}

}  // namespace gps
