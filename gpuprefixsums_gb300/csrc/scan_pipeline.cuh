// Persistent, warp-specialised tile-scan kernel for sm_103a.
//
// One CTA = W consumer warps + 1 producer warp. The producer's lane 0 takes
// tile ids (an atomic counter for chained scan, a static stride for
// reduce-then-scan), moves each tile global -> shared with one bulk copy
// (cp.async.bulk, completion on an mbarrier), and once the consumers have
// written the scanned tile back into the same shared buffer, moves it
// shared -> global with one bulk store. S shared buffers form a ring, so
// loads of the next tiles are in flight while the consumers scan and while
// the tile prefix is resolved.
//
// Consumers: each thread owns 64 contiguous bytes of the tile (16 u32 or
// 8 u64), read as four 16-byte chunks in a per-thread rotated order so that
// every quarter-warp touches all 32 banks exactly once. A thread reduces its
// items, a shuffle scan combines the threads of a warp, warp totals are
// combined through shared memory, and the tile's exclusive prefix comes
// either from the decoupled lookback over the tile descriptors
// (ChainedScanDecoupledLookback.cuh:50-77 does the same job with a 30-bit
// payload; here the payload is the full 32/64-bit value, tagged with a
// launch epoch) or from the spine array of a reduce-then-scan
// (ReduceThenScan.cuh:134-136).
//
// Every wait is bounded by the plan's budget (global timer); on expiry the
// kernel records a flag in the workspace header and keeps going without
// hanging, and the host reports GPS_ERR_TIMEOUT.
#pragma once
#include <cstdint>

#include "gps_internal.h"
#include "gps_ptx.cuh"

namespace gps {

constexpr uint32_t kFullMask = 0xFFFFFFFFu;

// ------------------------------------------------------ descriptor traits
template <typename T>
struct DescTraits;

// u32: one 64-bit word = status:2 | epoch:30 | value:32.
template <>
struct DescTraits<uint32_t> {
    using word = uint64_t;
    __device__ static word pack(uint32_t status, uint32_t epoch, uint32_t v) {
        return (static_cast<uint64_t>(status) << 62) |
               (static_cast<uint64_t>(epoch & kEpochMask) << 32) | v;
    }
    __device__ static word load(const word* p) { return ptx::ld_relaxed_u64(p); }
    __device__ static void store(word* p, word w) { ptx::st_relaxed_u64(p, w); }
    __device__ static word cas(word* p, word cmp, word val) { return ptx::atom_cas_u64(p, cmp, val); }
    __device__ static uint32_t status(word w, uint32_t epoch) {
        return (static_cast<uint32_t>(w >> 32) & kEpochMask) == (epoch & kEpochMask)
                   ? static_cast<uint32_t>(w >> 62)
                   : kNotReady;
    }
    __device__ static uint32_t value(word w) { return static_cast<uint32_t>(w); }
    __device__ static bool same(word a, word b) { return a == b; }
    __device__ static word zero() { return 0; }
    __device__ static word shfl(word w, uint32_t src) { return __shfl_sync(0xFFFFFFFFu, w, src); }
};

// u64: one 128-bit word = {lo: value, hi: status:2 | 32 zero bits | epoch:30}.
template <>
struct DescTraits<uint64_t> {
    using word = ptx::u64x2;
    __device__ static word pack(uint32_t status, uint32_t epoch, uint64_t v) {
        word w;
        w.lo = v;
        w.hi = (static_cast<uint64_t>(status) << 62) | (epoch & kEpochMask);
        return w;
    }
    __device__ static word load(const word* p) { return ptx::ld_relaxed_b128(p); }
    __device__ static void store(word* p, word w) { ptx::st_relaxed_b128(p, w); }
    __device__ static word cas(word* p, word cmp, word val) { return ptx::atom_cas_b128(p, cmp, val); }
    __device__ static uint32_t status(word w, uint32_t epoch) {
        return (static_cast<uint32_t>(w.hi) & kEpochMask) == (epoch & kEpochMask)
                   ? static_cast<uint32_t>(w.hi >> 62)
                   : kNotReady;
    }
    __device__ static uint64_t value(word w) { return w.lo; }
    __device__ static bool same(word a, word b) { return a.lo == b.lo && a.hi == b.hi; }
    __device__ static word zero() { return word{0, 0}; }
    __device__ static word shfl(word w, uint32_t src) {
        word r;
        r.lo = __shfl_sync(0xFFFFFFFFu, w.lo, src);
        r.hi = __shfl_sync(0xFFFFFFFFu, w.hi, src);
        return r;
    }
};

// ------------------------------------------------------------ warp helpers
template <typename T>
__device__ __forceinline__ T warp_inclusive_scan(T x, uint32_t lane) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const T y = __shfl_up_sync(kFullMask, x, d);
        if (lane >= static_cast<uint32_t>(d)) x += y;
    }
    return x;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T x) {
#pragma unroll
    for (int m = 16; m; m >>= 1) x += __shfl_xor_sync(kFullMask, x, m);
    return x;
}

__device__ __forceinline__ bool named_bar_or(uint32_t id, uint32_t threads, bool pred) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.or.pred q, %2, %3, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"(static_cast<uint32_t>(pred)), "r"(id), "r"(threads)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ uint32_t ld_volatile_u32(const uint32_t* p) {
    return *reinterpret_cast<const volatile uint32_t*>(p);
}

__device__ __forceinline__ void raise_error(WsHeader* hdr, uint32_t flag) {
    atomicOr(&hdr->error_flags, flag);
}

__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    // Murmur3 finaliser; selects stalled tiles in mode 2.
    x ^= x >> 16;
    x *= 0x85ebca6bu;
    x ^= x >> 13;
    x *= 0xc2b2ae35u;
    x ^= x >> 16;
    return x;
}

__device__ __forceinline__ bool tile_is_stalled(const StallConfig& sc, uint32_t t) {
    if (sc.mode == 1) return sc.period != 0 && (t % sc.period) == 0;
    if (sc.mode == 2) return sc.period != 0 && (mix32(t * 0x9E3779B9u ^ sc.seed) % sc.period) == 0;
    return false;
}

// Number of valid elements in tile t.
template <int TILE>
__device__ __forceinline__ uint32_t tile_count(uint64_t n, uint32_t t) {
    const uint64_t start = static_cast<uint64_t>(t) * TILE;
    const uint64_t rem = n - start;
    return rem < static_cast<uint64_t>(TILE) ? static_cast<uint32_t>(rem) : static_cast<uint32_t>(TILE);
}

// --------------------------------------------------- fallback re-reduction
// Warp-wide sum of the input of tile `t` read straight from global memory;
// used when a predecessor withholds its aggregate (Decoupled Fallback,
// EmulatedDeadlocking.cuh:113-133).
template <typename T, int TILE>
__device__ T warp_reduce_tile_input(const T* in, uint64_t n, uint32_t t, uint32_t lane) {
    const uint64_t start = static_cast<uint64_t>(t) * TILE;
    const uint32_t cnt = tile_count<TILE>(n, t);
    T acc = 0;
    for (uint32_t i = lane; i < cnt; i += 32) acc += in[start + i];
    return warp_sum(acc);
}

// ------------------------------------------------------------- lookback
// Run by one whole warp for tile t > 0. Returns the sum of all tiles before t
// (mod 2^w). Lane l of each window reads the descriptor of tile base-l; the
// nearest inclusive prefix ends the walk, a fully aggregated window moves it
// 32 tiles back. Bounded by the wait budget.
template <typename T, int TILE, bool STALL>
__device__ T lookback(const ScanArgs& a, uint32_t t, uint32_t epoch, uint32_t lane, T carry) {
    using D = DescTraits<T>;
    using word = typename D::word;
    word* desc = static_cast<word*>(a.desc);
    T prefix = 0;
    int64_t base = static_cast<int64_t>(t) - 1;
    uint32_t polls = 0;
    uint64_t deadline = 0;
    while (true) {
        const int64_t idx = base - static_cast<int64_t>(lane);
        word w = D::zero();
        uint32_t st = kInclusive;
        T val = 0;
        if (idx >= 0) {
            w = D::load(desc + idx);
            st = D::status(w, epoch);
            val = static_cast<T>(D::value(w));
        }
        const uint32_t vb = __ballot_sync(kFullMask, st != kNotReady);
        const uint32_t ib = __ballot_sync(kFullMask, st == kInclusive);
        if (ib) {
            const uint32_t first = __ffs(ib) - 1;
            const uint32_t need = first == 31 ? kFullMask : ((2u << first) - 1u);
            if ((vb & need) == need) {
                prefix += warp_sum(lane <= first ? val : T(0));
                return prefix;
            }
        } else if (vb == kFullMask) {
            prefix += warp_sum(val);
            base -= 32;
            polls = 0;
            continue;
        }
        // Window not resolvable yet.
        ++polls;
        if (STALL) {
            if (lane == 0) atomicAdd(&a.hdr->stat_polls, 1ull);
            if (a.stall.fallback_polls != 0 && polls >= a.stall.fallback_polls) {
                // Re-reduce the nearest predecessor that is still not ready and
                // try to insert its aggregate.
                const uint32_t f = __ffs(~vb) - 1;
                const int64_t fidx = base - static_cast<int64_t>(f);
                const word seen = D::shfl(w, f);
                const T agg = warp_reduce_tile_input<T, TILE>(static_cast<const T*>(a.in), a.n,
                                                             static_cast<uint32_t>(fidx), lane);
                if (lane == 0) {
                    __threadfence();
                    const word nw = fidx == 0 ? D::pack(kInclusive, epoch, carry + agg) : D::pack(kAggregate, epoch, agg);
                    const word old = D::cas(desc + fidx, seen, nw);
                    atomicAdd(&a.hdr->stat_fallbacks, 1ull);
                    if (D::same(old, seen)) atomicAdd(&a.hdr->stat_inserts, 1ull);
                }
                __syncwarp();
                polls = 0;
                continue;
            }
        }
        if ((polls & 31u) == 1u) {
            const uint64_t now = ptx::global_timer_ns();
            if (deadline == 0) deadline = now + a.wait_budget_ns;
            bool give_up = now > deadline || ld_volatile_u32(&a.hdr->error_flags) != 0;
            give_up = __shfl_sync(kFullMask, give_up, 0);
            if (give_up) {
                if (lane == 0) raise_error(a.hdr, kErrLookbackTimeout);
                return prefix;
            }
        }
    }
}

// ----------------------------------------------------------- shared state
template <typename T, int W, int S>
struct PipeCtrl {
    uint64_t full[S];   // producer -> consumers: tile landed in shared memory
    uint64_t done[S];   // consumers -> producer: scanned tile written back
    uint32_t tile_of[S];
    T warp_tot[2][W];   // inclusive warp totals, double-buffered by iteration
    T tile_prefix[2];
};

template <typename T, int W, int S>
constexpr size_t pipeline_smem_bytes() {
    return static_cast<size_t>(S) * TileShape<T, W>::kTile * sizeof(T) + sizeof(PipeCtrl<T, W, S>);
}

// A 16-byte chunk of elements.
template <typename T>
struct __align__(16) Chunk {
    T v[16 / sizeof(T)];
};

// ------------------------------------------------------------------ kernel
template <typename T, int W, int S, bool INCL, bool BULK, PrefixMode PM, bool STALL>
__global__ void __launch_bounds__(TileShape<T, W>::kThreads)
    scan_pipeline_kernel(const ScanArgs a) {
    using Shape = TileShape<T, W>;
    constexpr int TILE = Shape::kTile;
    constexpr int ITEMS = Shape::kItems;
    constexpr int EPC = 16 / static_cast<int>(sizeof(T));  // elements per chunk
    constexpr int CHUNKS = ITEMS / EPC;                      // == 4
    constexpr uint32_t NCONS = Shape::kConsumers;
    static_assert(CHUNKS == 4, "rotation scheme assumes four 16-byte chunks per thread");
    using D = DescTraits<T>;
    using word = typename D::word;

    extern __shared__ __align__(1024) uint8_t smem_raw[];
    T* bufs = reinterpret_cast<T*>(smem_raw);
    auto* ctrl = reinterpret_cast<PipeCtrl<T, W, S>*>(smem_raw + static_cast<size_t>(S) * TILE * sizeof(T));

    const uint32_t tid = threadIdx.x;
    const uint32_t warp = tid >> 5;
    const uint32_t lane = tid & 31u;

    if (tid == 0) {
#pragma unroll
        for (int s = 0; s < S; ++s) {
            ptx::mbar_init(&ctrl->full[s], 1);
            ptx::mbar_init(&ctrl->done[s], W);
        }
        ptx::fence_mbar_init();
    }
    __syncthreads();

    const uint32_t epoch = (PM == PrefixMode::Lookback) ? ld_volatile_u32(&a.hdr->epoch) : 0u;

    // ======================================================== producer warp
    if (warp == W) {
        if (lane != 0) return;
        bool stop = false;
        uint64_t k_static = 0;
        auto next_tile = [&]() -> uint32_t {
            if (stop) return kTileEnd;
            uint64_t t;
            if (PM == PrefixMode::Spine) {
                t = blockIdx.x + k_static * gridDim.x;
                ++k_static;
            } else {
                if (ld_volatile_u32(&a.hdr->error_flags) != 0) {
                    stop = true;
                    return kTileEnd;
                }
                t = atomicAdd(&a.hdr->tile_counter, 1u);
            }
            if (t >= a.num_tiles) {
                stop = true;
                return kTileEnd;
            }
            return static_cast<uint32_t>(t);
        };
        auto issue = [&](int s, uint32_t t) {
            ctrl->tile_of[s] = t;
            if (BULK && t != kTileEnd) {
                const uint32_t bytes = (tile_count<TILE>(a.n, t) * static_cast<uint32_t>(sizeof(T))) & ~15u;
                ptx::mbar_arrive_expect_tx(&ctrl->full[s], bytes);
                if (bytes)
                    ptx::bulk_load(bufs + static_cast<size_t>(s) * TILE,
                                   static_cast<const T*>(a.in) + static_cast<uint64_t>(t) * TILE, bytes,
                                   &ctrl->full[s]);
            } else {
                ptx::mbar_arrive(&ctrl->full[s]);
            }
        };
#pragma unroll
        for (int s = 0; s < S; ++s) issue(s, next_tile());

        const uint64_t budget = a.wait_budget_ns * 4 + 1000000000ull;
        for (uint32_t it = 0;; ++it) {
            const int s = static_cast<int>(it % S);
            const uint32_t ph = (it / S) & 1u;
            const uint32_t t = ctrl->tile_of[s];
            if (t == kTileEnd) break;
            if (!ptx::mbar_try_wait(&ctrl->done[s], ph)) {
                const uint64_t deadline = ptx::global_timer_ns() + budget;
                if (!ptx::mbar_wait_bounded(&ctrl->done[s], ph, deadline)) {
                    raise_error(a.hdr, kErrPipelineTimeout);
                    break;
                }
            }
            if (BULK) {
                const uint32_t bytes = (tile_count<TILE>(a.n, t) * static_cast<uint32_t>(sizeof(T))) & ~15u;
                if (bytes)
                    ptx::bulk_store(static_cast<T*>(a.out) + static_cast<uint64_t>(t) * TILE,
                                    bufs + static_cast<size_t>(s) * TILE, bytes);
                ptx::bulk_commit();
            }
            if (it >= 1) {
                const int ps = static_cast<int>((it - 1) % S);
                if (BULK) ptx::bulk_wait_read<1>();
                issue(ps, next_tile());
            }
        }
        if (BULK) ptx::bulk_wait_all<0>();

        if (PM == PrefixMode::Lookback) {
            // The last CTA out returns the counters to zero and advances the
            // epoch, which retires every descriptor of this launch.
            __threadfence();
            const uint32_t prev = atomicAdd(&a.hdr->exit_counter, 1u);
            if (prev == gridDim.x - 1) {
                __threadfence();
                a.hdr->tile_counter = 0;
                a.hdr->exit_counter = 0;
                uint32_t e = epoch + 1;
                if ((e & kEpochMask) == 0) {
                    word* desc = static_cast<word*>(a.desc);
                    for (unsigned long long i = 0; i < a.hdr->capacity_tiles; ++i) D::store(desc + i, D::zero());
                    e += 1;
                }
                __threadfence();
                a.hdr->epoch = e;
            }
        }
        return;
    }

    // ======================================================== consumer warps
    const uint32_t rot = (tid >> 1) & 3u;  // per-thread chunk rotation
    // Value added to every output (the running total of earlier chunks when a
    // long host array is scanned piece by piece).
    const T carry = a.carry_in != nullptr ? *static_cast<const T*>(a.carry_in) : T(0);
    const uint64_t mbar_budget = a.wait_budget_ns;

    for (uint32_t it = 0;; ++it) {
        const int s = static_cast<int>(it % S);
        const uint32_t ph = (it / S) & 1u;
        const uint32_t par = it & 1u;
        bool ok = ptx::mbar_try_wait(&ctrl->full[s], ph);
        if (!ok) ok = ptx::mbar_wait_bounded(&ctrl->full[s], ph, ptx::global_timer_ns() + mbar_budget);
        const uint32_t t = ctrl->tile_of[s];
        T* sb = bufs + static_cast<size_t>(s) * TILE;
        const bool live = ok && t != kTileEnd;
        const uint32_t cnt = live ? tile_count<TILE>(a.n, t) : 0u;
        const bool full_tile = BULK && cnt == static_cast<uint32_t>(TILE);
        const uint64_t gbase = static_cast<uint64_t>(live ? t : 0u) * TILE;
        const uint32_t bulk_elems = BULK ? ((cnt * static_cast<uint32_t>(sizeof(T))) & ~15u) / sizeof(T) : 0u;

        // ---- load my 64 bytes, in rotated chunk order
        T v[ITEMS];
        if (full_tile) {
#pragma unroll
            for (int j = 0; j < CHUNKS; ++j) {
                const uint32_t c = (j + rot) & 3u;
                const Chunk<T> q = *reinterpret_cast<const Chunk<T>*>(sb + tid * ITEMS + c * EPC);
#pragma unroll
                for (int e = 0; e < EPC; ++e) v[j * EPC + e] = q.v[e];
            }
        } else {
#pragma unroll
            for (int j = 0; j < CHUNKS; ++j) {
                const uint32_t c = (j + rot) & 3u;
#pragma unroll
                for (int e = 0; e < EPC; ++e) {
                    const uint32_t li = tid * ITEMS + c * EPC + e;
                    T x = 0;
                    if (li < bulk_elems)
                        x = sb[li];
                    else if (li < cnt)
                        x = static_cast<const T*>(a.in)[gbase + li];
                    v[j * EPC + e] = x;
                }
            }
        }

        // ---- thread level: chunk sums and the logical prefix of each chunk
        T cs[CHUNKS];
#pragma unroll
        for (int j = 0; j < CHUNKS; ++j) {
            T x = v[j * EPC];
#pragma unroll
            for (int e = 1; e < EPC; ++e) x += v[j * EPC + e];
            cs[j] = x;
        }
        const T q1 = cs[0];
        const T q2 = q1 + cs[1];
        const T q3 = q2 + cs[2];
        const T thread_total = q3 + cs[3];
        // Register j holds logical chunk (j + rot) & 3; the chunk-0 register
        // is (4 - rot) & 3. Exclusive prefix of register j in logical order:
        // Q[j] - Q[start] (+ total when register j wraps before start).
        const T qstart = rot == 0 ? T(0) : (rot == 1 ? q3 : (rot == 2 ? q2 : q1));
        T cpre[CHUNKS];
        {
            const T qj[4] = {T(0), q1, q2, q3};
#pragma unroll
            for (int j = 0; j < CHUNKS; ++j) {
                const bool wraps = rot != 0 && (j + rot) < 4u;
                cpre[j] = qj[j] - qstart + (wraps ? thread_total : T(0));
            }
        }

        // ---- warp level
        const T winc = warp_inclusive_scan(thread_total, lane);
        const T wexc = winc - thread_total;
        if (lane == 31) ctrl->warp_tot[par][warp] = winc;

        // Barrier A, which also agrees on "stop" (a timed-out wait or end).
        const bool stop = named_bar_or(1, NCONS, !live);
        if (stop) {
            if (!ok && lane == 0 && warp == 0) raise_error(a.hdr, kErrPipelineTimeout);
            break;
        }

        // ---- block level: this warp's prefix and the tile aggregate
        T wpre = 0, agg = 0;
#pragma unroll
        for (int w2 = 0; w2 < W; ++w2) {
            const T x = ctrl->warp_tot[par][w2];
            wpre += (static_cast<uint32_t>(w2) < warp) ? x : T(0);
            agg += x;
        }

        T tile_prefix;
        if (PM == PrefixMode::Spine) {
            tile_prefix = carry + (t == 0 ? T(0) : static_cast<const T*>(a.spine)[t - 1]);
            if (a.carry_out != nullptr && t == a.num_tiles - 1 && tid == 0)
                *static_cast<T*>(a.carry_out) = tile_prefix + agg;
        } else {
            if (warp == 0) {
                word* desc = static_cast<word*>(a.desc);
                T pre = carry;
                if (lane == 0) {
                    bool publish = true;
                    if (STALL && tile_is_stalled(a.stall, t)) {
                        // Withhold the aggregate until the delay ends or a
                        // successor inserts it (EmulatedDeadlocking.cuh:64-70).
                        atomicAdd(&a.hdr->stat_stalls, 1ull);
                        const uint64_t until = ptx::global_timer_ns() + a.stall.delay_ns;
                        while (true) {
                            const word seen = D::load(desc + t);
                            if (D::status(seen, epoch) != kNotReady) {
                                publish = false;
                                break;
                            }
                            if (ptx::global_timer_ns() > until) break;
                            __nanosleep(200);
                        }
                    }
                    // A rescuer computes the same integer aggregate, so a plain
                    // store over an inserted one is harmless; rescuers use a
                    // CAS so that they never overwrite an inclusive prefix.
                    if (publish)
                        D::store(desc + t, D::pack(t == 0 ? kInclusive : kAggregate, epoch, carry + agg));
                }
                __syncwarp();
                if (t != 0) {
                    pre = lookback<T, TILE, STALL>(a, t, epoch, lane, carry);
                    if (lane == 0) D::store(desc + t, D::pack(kInclusive, epoch, pre + agg));
                }
                if (lane == 0) {
                    ctrl->tile_prefix[par] = pre;
                    if (a.carry_out != nullptr && t == a.num_tiles - 1) *static_cast<T*>(a.carry_out) = pre + agg;
                }
                if (STALL) __threadfence();
            }
            ptx::named_bar_sync(1, NCONS);  // barrier B
            tile_prefix = ctrl->tile_prefix[par];
        }

        // ---- outputs
        const T base = tile_prefix + wpre + wexc;
#pragma unroll
        for (int j = 0; j < CHUNKS; ++j) {
            T run = base + cpre[j];
#pragma unroll
            for (int e = 0; e < EPC; ++e) {
                const T x = v[j * EPC + e];
                if (INCL) {
                    run += x;
                    v[j * EPC + e] = run;
                } else {
                    v[j * EPC + e] = run;
                    run += x;
                }
            }
        }
        if (full_tile) {
#pragma unroll
            for (int j = 0; j < CHUNKS; ++j) {
                const uint32_t c = (j + rot) & 3u;
                Chunk<T> q;
#pragma unroll
                for (int e = 0; e < EPC; ++e) q.v[e] = v[j * EPC + e];
                *reinterpret_cast<Chunk<T>*>(sb + tid * ITEMS + c * EPC) = q;
            }
        } else {
#pragma unroll
            for (int j = 0; j < CHUNKS; ++j) {
                const uint32_t c = (j + rot) & 3u;
#pragma unroll
                for (int e = 0; e < EPC; ++e) {
                    const uint32_t li = tid * ITEMS + c * EPC + e;
                    if (li < bulk_elems)
                        sb[li] = v[j * EPC + e];
                    else if (li < cnt)
                        static_cast<T*>(a.out)[gbase + li] = v[j * EPC + e];
                }
            }
        }
        if (BULK) ptx::fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) ptx::mbar_arrive(&ctrl->done[s]);
    }
}

}  // namespace gps
