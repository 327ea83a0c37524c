// Reduce-then-scan for u32 and u64: three launches, as in the reference's
// ReduceThenScanDispatcher::DispatchKernels{Ex,In}clusive
// (GPUPrefixSumsCUDA/ReduceThenScanDispatcher.cuh:165-187):
//   1. reduce: one CTA per tile writes the tile's sum
//      (ReduceThenScan::Reduce, ReduceThenScan.cuh:15-53);
//   2. spine: one 1024-thread CTA scans the tile sums in place, inclusive
//      (ReduceThenScan::SpineScan, ReduceThenScan.cuh:56-104);
//   3. propagate: re-reads every tile, scans it and adds the spine value of
//      the previous tile (ReduceThenScan::Propagate, ReduceThenScan.cuh:106-161),
//      here the same bulk-copy pipeline kernel as the chained scan, fed from
//      the spine instead of the lookback.
// It reads the input twice (12 bytes per u32 element against 8 for the
// single-pass scan) and keeps no inter-CTA waits.
#include "launch_util.h"
#include "scan_pipeline.cuh"

namespace gps {

namespace {

constexpr int kRtsWarps = 4;
constexpr int kRtsStages = 6;
constexpr int kReduceThreads = 256;
constexpr int kSpineThreads = 1024;
constexpr int kSpineItems = 8;

template <typename T>
__global__ void __launch_bounds__(kReduceThreads)
    rts_reduce_kernel(const T* __restrict__ in, uint64_t n, T* __restrict__ tile_sums, uint32_t num_tiles,
                      bool vec_ok) {
    constexpr int TILE = TileShape<T, kRtsWarps>::kTile;
    constexpr int EPC = 16 / static_cast<int>(sizeof(T));
    constexpr int CHUNKS_PER_THREAD = TILE / EPC / kReduceThreads;
    __shared__ T warp_sums[kReduceThreads / 32];
    const uint32_t t = blockIdx.x;
    const uint64_t base = static_cast<uint64_t>(t) * TILE;
    const uint32_t cnt = tile_count<TILE>(n, t);
    T acc = 0;
    if (vec_ok && cnt == static_cast<uint32_t>(TILE)) {
        const Chunk<T>* src = reinterpret_cast<const Chunk<T>*>(in + base);
        Chunk<T> q[CHUNKS_PER_THREAD];
#pragma unroll
        for (int k = 0; k < CHUNKS_PER_THREAD; ++k) {
            const uint4 r = ptx::ld_stream_v4(src + threadIdx.x + k * kReduceThreads);
            q[k] = *reinterpret_cast<const Chunk<T>*>(&r);
        }
#pragma unroll
        for (int k = 0; k < CHUNKS_PER_THREAD; ++k)
#pragma unroll
            for (int e = 0; e < EPC; ++e) acc += q[k].v[e];
    } else {
        for (uint32_t i = threadIdx.x; i < cnt; i += kReduceThreads) acc += in[base + i];
    }
    acc = warp_sum(acc);
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    if (lane == 0) warp_sums[warp] = acc;
    __syncthreads();
    if (warp == 0) {
        T x = lane < kReduceThreads / 32 ? warp_sums[lane] : T(0);
        x = warp_sum(x);
        if (lane == 0) tile_sums[t] = x;
    }
}

// Inclusive scan of m tile sums in place by a single CTA, kSpineItems
// consecutive sums per thread per pass.
template <typename T>
__global__ void __launch_bounds__(kSpineThreads) rts_spine_kernel(T* sums, uint32_t m) {
    __shared__ T warp_tot[kSpineThreads / 32];
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    T carry = 0;
    for (uint64_t pass = 0; pass < m; pass += static_cast<uint64_t>(kSpineThreads) * kSpineItems) {
        T v[kSpineItems];
        T run = 0;
#pragma unroll
        for (int i = 0; i < kSpineItems; ++i) {
            const uint64_t idx = pass + static_cast<uint64_t>(tid) * kSpineItems + i;
            const T x = idx < m ? sums[idx] : T(0);
            run += x;
            v[i] = run;
        }
        const T winc = warp_inclusive_scan(run, lane);
        if (lane == 31) warp_tot[warp] = winc;
        __syncthreads();
        if (warp == 0) warp_tot[lane] = warp_inclusive_scan(warp_tot[lane], lane);
        __syncthreads();
        const T pre = carry + (warp ? warp_tot[warp - 1] : T(0)) + (winc - run);
#pragma unroll
        for (int i = 0; i < kSpineItems; ++i) {
            const uint64_t idx = pass + static_cast<uint64_t>(tid) * kSpineItems + i;
            if (idx < m) sums[idx] = pre + v[i];
        }
        carry += warp_tot[kSpineThreads / 32 - 1];
        __syncthreads();
    }
}

template <typename T, bool INCL, bool BULK>
cudaError_t launch_propagate(const ScanArgs& a, int num_sms, cudaStream_t stream, LaunchInfo* info) {
    using Shape = TileShape<T, kRtsWarps>;
    auto kern = scan_pipeline_kernel<T, kRtsWarps, kRtsStages, 1, INCL, BULK, PrefixMode::Spine, false>;
    constexpr size_t smem = pipeline_smem_bytes<T, kRtsWarps, kRtsStages>();
    int occ = 0;
    cudaError_t err = resident_ctas_per_sm(kern, Shape::kThreads, smem, &occ);
    if (err != cudaSuccess) return err;
    const int grid = persistent_grid(a.num_tiles, occ, num_sms);
    if (info) *info = LaunchInfo{grid, Shape::kThreads, smem};
    kern<<<grid, Shape::kThreads, smem, stream>>>(a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t dispatch_rts(bool inclusive, const ScanArgs& a0, void* tile_sums, int num_sms, cudaStream_t stream,
                         LaunchInfo* info) {
    const bool bulk = ((reinterpret_cast<uintptr_t>(a0.in) | reinterpret_cast<uintptr_t>(a0.out)) & 15u) == 0;
    const bool in_vec = (reinterpret_cast<uintptr_t>(a0.in) & 15u) == 0;
    T* sums = static_cast<T*>(tile_sums);
    rts_reduce_kernel<T><<<a0.num_tiles, kReduceThreads, 0, stream>>>(static_cast<const T*>(a0.in), a0.n, sums,
                                                                      a0.num_tiles, in_vec);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    rts_spine_kernel<T><<<1, kSpineThreads, 0, stream>>>(sums, a0.num_tiles);
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    ScanArgs a = a0;
    a.spine = sums;
    if (bulk)
        return inclusive ? launch_propagate<T, true, true>(a, num_sms, stream, info)
                         : launch_propagate<T, false, true>(a, num_sms, stream, info);
    return inclusive ? launch_propagate<T, true, false>(a, num_sms, stream, info)
                     : launch_propagate<T, false, false>(a, num_sms, stream, info);
}

}  // namespace

uint32_t rts_tile_elems(gps_dtype dtype) {
    return dtype == GPS_DTYPE_U64 ? TileShape<uint64_t, kRtsWarps>::kTile : TileShape<uint32_t, kRtsWarps>::kTile;
}

cudaError_t launch_rts(gps_dtype dtype, bool inclusive, const ScanArgs& a, void* tile_sums, int num_sms,
                       cudaStream_t stream, LaunchInfo* info) {
    if (dtype == GPS_DTYPE_U64) return dispatch_rts<uint64_t>(inclusive, a, tile_sums, num_sms, stream, info);
    return dispatch_rts<uint32_t>(inclusive, a, tile_sums, num_sms, stream, info);
}

}  // namespace gps
