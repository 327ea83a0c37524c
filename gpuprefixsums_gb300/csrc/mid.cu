// Single-pass chained scan for mid-size inputs: one 16 KB tile per CTA.
//
// The persistent L2-buffered kernel (scan_l2.cuh) pays a pipeline latency of
// about 10 us per launch (unit claim, HBM load, reduce, lookback, reload from
// L2, scan, store), which dominates at small sizes. Here every tile gets its
// own CTA of 256 threads, as in the reference's single-pass kernel
// (ChainedScanDecoupledLookback.cuh:79-139):
//   1. the tile id is the block index: a CTA waits only on lower block
//      indices, which the hardware dispatches first (CUB's decoupled
//      lookback relies on the same order); every wait is bounded, so a
//      violation would surface as GPS_ERR_TIMEOUT, never as a hang;
//   2. load the tile and block-scan it;
//   3. publish the tile aggregate and look back (warp 0): over the tiles of
//      its group of 32, then, if needed, over the descriptors of earlier
//      groups;
//   4. publish the inclusive prefix, add the prefix, store.
// The kernels keep their descriptors in a region of the plan of their own,
// tagged with the launch's grid id (%gridid: a 64-bit number the driver gives
// every grid launched in a CUDA context, graph replays included). A
// descriptor counts only when its tag is the current launch's, so a launch
// needs neither a clearing memset nor an end-of-launch retirement (the last
// CTA resetting counters and advancing an epoch): no atomic and no fence on
// any CTA's path.
#include "gps_device.cuh"
#include "gps_internal.h"
#include "launch_util.h"
#include "scan_pipeline.cuh"

namespace gps {
namespace {

constexpr int kMidThreads = 256;
// Resident CTAs per SM the aligned-buffer kernel is compiled for.
constexpr int kMidVecCtasPerSm = 8;

// ------------------------------------------------------------ descriptors
// One 16-byte word per tile: {lo: the value (u32 or u64), hi: status:2 |
// grid id:62}. Zeroed memory reads "not ready". 2^62 launches would have to
// pass in one context before a stale tag could come round again. Tile t's
// word is word t * a.desc_stride of the region: launches of more than one
// group of tiles give each tile a 128-byte line of its own, since tiles that
// publish while others read the same line waited up to 3 us for a read.
// Group descriptors always have a line each (word g * kMidDescStride).
constexpr uint64_t kGidMask = (1ull << 62) - 1;

struct MidDesc {
    __device__ static ptx::u64x2 pack(uint32_t status, uint64_t gid, uint64_t v) {
        ptx::u64x2 w;
        w.lo = v;
        w.hi = (static_cast<uint64_t>(status) << 62) | (gid & kGidMask);
        return w;
    }
    __device__ static uint32_t status(const ptx::u64x2& w, uint64_t gid) {
        return (w.hi & kGidMask) == (gid & kGidMask) ? static_cast<uint32_t>(w.hi >> 62) : kNotReady;
    }
};

__device__ __forceinline__ uint64_t grid_id() {
    uint64_t g;
    asm volatile("mov.u64 %0, %%gridid;" : "=l"(g));
    return g;
}

// ------------------------------------------------------- two-level lookback
// Tiles form groups of 32. Besides its tile descriptor, the last tile of each
// group publishes a group descriptor: the group's aggregate as soon as its
// in-group lookback is done, and the inclusive prefix through the group once
// its prefix is known. Warp 0 of a tile sums its in-group predecessors back to
// the nearest inclusive one (one descriptor per lane) and, when none of them
// is inclusive, adds the prefix of its group: a decoupled lookback over the
// group descriptors, 32 per poll. Each tile reads at most 31 tile descriptors
// and the group descriptors back to the nearest inclusive one. A flat
// lookback, in which every tile reads its predecessors' descriptors directly
// (one warp, or all warps of the CTA, 128 to 1024 per poll), measured slower
// from 2^19 elements on: all CTAs of a launch look back at once, and their
// reads, quadratic in the tile count, queue on the few L2 lines that hold the
// descriptors.
constexpr uint32_t kGroupTiles = 32;

struct LookbackSmem {
    uint32_t found;    // an inclusive tile was found in the group
    uint32_t timeout;  // a wait ran past its budget
};

// Warp-level lookback over the 32 descriptors at and below `top` (lane l reads
// slot top - l when it is at least `floor`). Polls until every slot from top
// down to the nearest inclusive one (or down to `floor`) is ready; returns
// whether an inclusive one was found and, in `sum`, the sum of those slots.
// Gives up after the wait budget, setting timed_out (then `sum` is 0).
template <typename T, uint32_t SPIN = 64>
__device__ bool warp_window(const ScanArgs& a, const ptx::u64x2* d, uint32_t stride, int64_t top, int64_t floor,
                            uint64_t gid, uint32_t lane, T& sum, bool& timed_out) {
    const int64_t idx = top - static_cast<int64_t>(lane);
    bool ready = idx < floor, incl = false;
    T v = 0;
    uint32_t polls = 0, backoff = 32;
    uint64_t deadline = 0;
    timed_out = false;
    while (true) {
        if (!ready) {
            const ptx::u64x2 w = ptx::ld_relaxed_b128(d + idx * stride);
            const uint32_t st = MidDesc::status(w, gid);
            if (st != kNotReady) {
                ready = true;
                v = static_cast<T>(w.lo);
                incl = st == kInclusive;
            }
        }
        const uint32_t inc_mask = __ballot_sync(kFullMask, incl);
        const uint32_t wait_mask = __ballot_sync(kFullMask, !ready);
        const uint32_t pinc = inc_mask ? static_cast<uint32_t>(__ffs(inc_mask) - 1) : 32u;
        const uint32_t need = pinc >= 31u ? kFullMask : (2u << pinc) - 1u;  // lanes 0 .. pinc
        if ((wait_mask & need) == 0) {
            sum = warp_sum(lane <= pinc ? v : T(0));
            return pinc != 32u;
        }
        ++polls;
        if ((polls & 15u) == 1u) {
            bool expired = false;
            if (lane == 0) {
                const uint64_t now = ptx::global_timer_ns();
                if (deadline == 0) deadline = now + a.wait_budget_ns;
                expired = now > deadline || ld_volatile_u32(&a.hdr->error_flags) != 0;
            }
            if (__shfl_sync(kFullMask, expired, 0)) {
                timed_out = true;
                sum = 0;
                return false;
            }
        }
        if (polls > SPIN) {
            __nanosleep(backoff);
            backoff = backoff < 1024 ? backoff * 2 : 1024;
        }
    }
}

// Publishes tile t's aggregate, resolves its exclusive prefix (carry_in for
// tile 0) and publishes its inclusive prefix; returns the prefix to every
// thread. `total` is the tile's sum, known to every thread. Warp 0 looks
// back; a barrier hands its result to the CTA.
template <typename T>
__device__ __forceinline__ T mid_tile_prefix(const ScanArgs& a, uint32_t t, uint64_t gid, T total, LookbackSmem& sm,
                                             T* s_pre) {
    ptx::u64x2* d1 = static_cast<ptx::u64x2*>(a.desc);
    ptx::u64x2* d2 = static_cast<ptx::u64x2*>(a.group_desc);
    const uint32_t s1 = a.desc_stride;
    const T carry = a.carry_in != nullptr ? *static_cast<const T*>(a.carry_in) : T(0);
    const uint32_t tid = threadIdx.x;
    const uint32_t g = t / kGroupTiles;
    const bool group_last = (t % kGroupTiles) == kGroupTiles - 1;
    if (t == 0) {
        if (tid == 0) {
            ptx::st_relaxed_b128(d1, MidDesc::pack(kInclusive, gid, static_cast<uint64_t>(carry + total)));
            if (a.carry_out != nullptr && a.num_tiles == 1) *static_cast<T*>(a.carry_out) = carry + total;
        }
        return carry;
    }
    if (tid < 32) {
        const uint32_t lane = tid;
        if (lane == 0)
            ptx::st_relaxed_b128(d1 + t * s1, MidDesc::pack(kAggregate, gid, static_cast<uint64_t>(total)));
        // The tiles of this group before t; tile 0 is inclusive, so group 0
        // always finds one.
        T in_sum;
        bool timed_out;
        const bool found = warp_window<T>(a, d1, s1, static_cast<int64_t>(t) - 1,
                                          static_cast<int64_t>(g) * kGroupTiles, gid, lane, in_sum, timed_out);
        if (lane == 0 && group_last && !timed_out)
            ptx::st_relaxed_b128(d2 + g * kMidDescStride, MidDesc::pack(found ? kInclusive : kAggregate, gid,
                                                       static_cast<uint64_t>(in_sum + total)));
        // No inclusive tile in the group before t: the prefix of the group, a
        // decoupled lookback over the group descriptors, 32 per poll.
        T gsum = 0;
        if (!found && !timed_out) {
            int64_t top = static_cast<int64_t>(g) - 1;
            while (true) {
                T part;
                const bool gf = warp_window<T>(a, d2, kMidDescStride, top, 0, gid, lane, part, timed_out);
                if (timed_out) break;
                gsum += part;
                if (gf || top < 32) break;  // group 0's descriptor is inclusive
                top -= 32;
            }
        }
        if (lane == 0) {
            s_pre[0] = in_sum + gsum;
            sm.timeout = timed_out ? 1u : 0u;
            sm.found = found ? 1u : 0u;
        }
    }
    __syncthreads();
    if (sm.timeout != 0) {
        if (tid == 0) raise_error(a.hdr, kErrLookbackTimeout);
        return T(0);
    }
    const T pre = s_pre[0];
    if (tid == 0) {
        ptx::st_relaxed_b128(d1 + t * s1, MidDesc::pack(kInclusive, gid, static_cast<uint64_t>(pre + total)));
        if (group_last && sm.found == 0)
            ptx::st_relaxed_b128(d2 + g * kMidDescStride, MidDesc::pack(kInclusive, gid, static_cast<uint64_t>(pre + total)));
        if (a.carry_out != nullptr && t == a.num_tiles - 1) *static_cast<T*>(a.carry_out) = pre + total;
    }
    return pre;
}

// Buffers not aligned to 16 bytes: each thread loads and stores its 64
// bytes element by element.
template <typename T, bool INCL>
__global__ void __launch_bounds__(kMidThreads, 2) mid_scan_kernel(const ScanArgs a) {
    constexpr int TILE = 16384 / static_cast<int>(sizeof(T));
    constexpr int ITEMS = TILE / kMidThreads;  // 16 u32 or 8 u64: 64 bytes
    __shared__ gps_device::BlockScanStorage<kMidThreads, T> st;
    __shared__ LookbackSmem lsm;
    __shared__ T s_pre[1];

    const uint32_t tid = threadIdx.x;
    const uint32_t t = blockIdx.x;
    const uint64_t gid = grid_id();
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
    T run = mid_tile_prefix<T>(a, t, gid, total, lsm, s_pre) + before;
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
}

// The same scan for 16-byte-aligned buffers. The tile is four rows of 256
// 16-byte chunks, and thread tid holds chunk tid of every row, so each warp
// load or store instruction covers 512 contiguous bytes. The exclusive prefix
// of chunk (r, tid) within the tile is the sum of the rows before r plus the
// chunks of row r before tid: the four chunk sums are warp-scanned together,
// the warp totals go through shared memory in row-major order (row r, warp
// w at r * 8 + w), and one warp scan of those 32 totals gives every (row,
// warp) its offset -- one barrier for the whole block scan. Chunks are read
// twice: for the sums, and after the lookback to scan and store them (the
// second read hits this SM's L1). Neither tile data nor chunk offsets stay in
// registers across the lookback, which keeps the kernel at 32 registers and
// eight CTAs per SM: on 152 SMs up to 1216 tiles (2^22 u32 elements fit) run
// in one wave. There is no shared-memory staging and no mbarrier to set up,
// so every CTA issues its loads as soon as it starts.
template <typename T, bool INCL>
__global__ void __launch_bounds__(kMidThreads, kMidVecCtasPerSm) mid_vec_kernel(const ScanArgs a) {
    constexpr int TILE = 16384 / static_cast<int>(sizeof(T));
    constexpr int EPC = 16 / static_cast<int>(sizeof(T));
    constexpr int ROW = kMidThreads * EPC;  // elements per row
    constexpr int ROWS = TILE / ROW;        // 4
    constexpr int WARPS = kMidThreads / 32;
    static_assert(ROWS * WARPS == 32, "one warp scans all (row, warp) totals");
    __shared__ T s_tot[ROWS * WARPS];
    __shared__ T s_off[ROWS][kMidThreads];  // chunk offsets, kept here across the lookback
    __shared__ LookbackSmem lsm;
    __shared__ T s_pre[1];

    const uint32_t tid = threadIdx.x;
    const uint32_t lane = tid & 31u;
    const uint32_t warp = tid >> 5;
    const uint32_t t = blockIdx.x;
    const uint64_t gid = grid_id();
    const uint64_t t0 = static_cast<uint64_t>(t) * TILE;
    // Elements of this tile; chunk (r, tid) starts at element r * ROW + tid * EPC.
    const uint32_t cnt = static_cast<uint32_t>(min(static_cast<uint64_t>(TILE), a.n - t0));
    const bool full = cnt == static_cast<uint32_t>(TILE);
    const T* src = static_cast<const T*>(a.in) + t0 + tid * EPC;
    T* dst = static_cast<T*>(a.out) + t0 + tid * EPC;

    T cs[ROWS];
    {
        Chunk<T> q[ROWS];
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
            const uint32_t off = r * ROW + tid * EPC;
            if (full || off + EPC <= cnt) {
                q[r] = *reinterpret_cast<const Chunk<T>*>(src + r * ROW);
            } else {
#pragma unroll
                for (int e = 0; e < EPC; ++e) q[r].v[e] = off + e < cnt ? src[r * ROW + e] : T(0);
            }
        }
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
            T x = 0;
#pragma unroll
            for (int e = 0; e < EPC; ++e) x += q[r].v[e];
            cs[r] = x;
        }
    }
    // Block scan of the four rows at once; each thread's four chunk offsets
    // wait in shared memory during the lookback.
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
        T wt;
        cs[r] = gps_device::warp_exclusive_scan<gps_device::WarpAlgo::KoggeStone>(cs[r], gps_device::Plus(), &wt);
        if (lane == 0) s_tot[r * WARPS + warp] = wt;
    }
    __syncthreads();
    T total;
    {
        const T x = s_tot[lane];
        const T xi = gps_device::warp_inclusive_scan<gps_device::WarpAlgo::KoggeStone>(x, gps_device::Plus());
        const T xe = xi - x;
        total = __shfl_sync(kFullMask, xi, 31);
#pragma unroll
        for (int r = 0; r < ROWS; ++r) s_off[r][tid] = cs[r] + __shfl_sync(kFullMask, xe, r * WARPS + warp);
    }

    const T base = mid_tile_prefix<T>(a, t, gid, total, lsm, s_pre);

    Chunk<T> q[ROWS];
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
        const uint32_t off = r * ROW + tid * EPC;
        if (full || off + EPC <= cnt) {
            q[r] = *reinterpret_cast<const Chunk<T>*>(src + r * ROW);
        } else {
#pragma unroll
            for (int e = 0; e < EPC; ++e) q[r].v[e] = off + e < cnt ? src[r * ROW + e] : T(0);
        }
    }
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
        const uint32_t off = r * ROW + tid * EPC;
        T acc = base + s_off[r][tid];
#pragma unroll
        for (int e = 0; e < EPC; ++e) {
            const T x = q[r].v[e];
            if (INCL) {
                acc += x;
                q[r].v[e] = acc;
            } else {
                q[r].v[e] = acc;
                acc += x;
            }
        }
        if (full || off + EPC <= cnt) {
            *reinterpret_cast<Chunk<T>*>(dst + r * ROW) = q[r];
        } else {
#pragma unroll
            for (int e = 0; e < EPC; ++e)
                if (off + e < cnt) dst[r * ROW + e] = q[r].v[e];
        }
    }
}

template <typename T, bool INCL, bool VEC>
cudaError_t launch_mid_v(const ScanArgs& a0, cudaStream_t stream, LaunchInfo* info) {
    auto kern = VEC ? mid_vec_kernel<T, INCL> : mid_scan_kernel<T, INCL>;
    ScanArgs a = a0;
    a.desc_stride = a.num_tiles > kGroupTiles && a.num_tiles <= kMidStrideMaxTiles ? kMidDescStride : 1u;
    const int grid = static_cast<int>(a.num_tiles);
    if (info) *info = LaunchInfo{grid, kMidThreads, 0};
    kern<<<grid, kMidThreads, 0, stream>>>(a);
    return cudaGetLastError();
}

template <typename T, bool INCL>
cudaError_t launch_mid_t(const ScanArgs& a, cudaStream_t stream, LaunchInfo* info) {
    if (((reinterpret_cast<uintptr_t>(a.desc) | reinterpret_cast<uintptr_t>(a.group_desc)) & 15u) != 0 ||
        a.desc == nullptr || a.group_desc == nullptr)
        return cudaErrorInvalidValue;
    const bool vec = ((reinterpret_cast<uintptr_t>(a.in) | reinterpret_cast<uintptr_t>(a.out)) & 15u) == 0;
    return vec ? launch_mid_v<T, INCL, true>(a, stream, info) : launch_mid_v<T, INCL, false>(a, stream, info);
}

}  // namespace

cudaError_t launch_mid(gps_dtype dtype, bool inclusive, const ScanArgs& a, int /*num_sms*/, cudaStream_t stream,
                       LaunchInfo* info) {
    if (dtype == GPS_DTYPE_U64)
        return inclusive ? launch_mid_t<uint64_t, true>(a, stream, info) : launch_mid_t<uint64_t, false>(a, stream, info);
    return inclusive ? launch_mid_t<uint32_t, true>(a, stream, info) : launch_mid_t<uint32_t, false>(a, stream, info);
}

}  // namespace gps
