// Persistent, warp-specialised tile-scan kernel for sm_103a.
//
// Each CTA runs a ring of S shared-memory stages, one 16 KB tile each, and
// four roles:
//   producer  (1 thread)  takes tile ids (an atomic counter for the chained
//             scan, a static stride for reduce-then-scan), moves each tile
//             global -> shared with one bulk copy (cp.async.bulk, completion
//             on an mbarrier) and, once it is scanned, shared -> global with
//             one bulk store;
//   reduce    (RW warps)  sums the landed tile, publishes its aggregate in the
//             tile descriptor and leaves each thread's offset in shared
//             memory;
//   lookback  (1 warp)    resolves the tile's exclusive prefix, in tile order:
//             decoupled lookback over the descriptors (the reference's
//             ChainedScanDecoupledLookback.cuh:50-77 does this with a 30-bit
//             payload; here the payload is the full 32/64-bit value, tagged
//             with a launch epoch) or the spine of a reduce-then-scan
//             (ReduceThenScan.cuh:134-136);
//   finalize  (RW warps)  adds prefix and offsets, writes the tile back.
//
// Every wait is bounded by the plan's budget (global timer); on expiry the
// kernel records a flag in the workspace header and winds down without
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

// Whether lookback unit u of num_units withholds its aggregate. The last unit
// never does: no successor exists to re-reduce it, so its stall would only
// burn the delay (the reference's stalled tiles spin until a successor
// rescues them, EmulatedDeadlocking.cuh:64-67, and it exempts a grid of one
// tile; a stalled last tile there never returns).
__device__ __forceinline__ bool unit_stalls(const StallConfig& sc, uint32_t u, uint32_t num_units) {
    return u + 1 < num_units && tile_is_stalled(sc, u);
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
// Descriptors read by each lane per poll: 128 bytes, i.e. 16 u32-scan
// descriptors or 8 u64-scan descriptors; a window is 32 lanes of that (512 or
// 256 slots).
template <typename W, int LANE_BYTES = 128>
constexpr int lookback_per_lane() {
    return LANE_BYTES / static_cast<int>(sizeof(W));
}

// Run by one whole warp for lookback unit u > 0 (a tile, or a group of SPAN
// consecutive elements). Returns the sum of all units before u (mod 2^w).
//
// `bound` is a unit before u whose inclusive prefix `bound_val` the caller
// already knows (its own previous unit), or -1: the walk never goes past it.
// A window is the 32*K descriptor slots ending at `top`; its 16-byte pairs are
// spread over the lanes so that each load instruction reads whole L2 lines.
// Each slot's distance from `top` is its position; the nearest inclusive
// prefix (smallest position, or the bound) ends the walk once every nearer
// slot holds an aggregate; a window of aggregates only moves it back by 32*K
// slots. Slots >= u count as empty aggregates. A poll that finds a needed
// slot not ready re-reads only the pairs holding such slots, after an
// exponential back-off (from poll SPIN on; the polls before it re-read at
// once). Bounded by the wait budget.
// LANE_BYTES (16 to 128) sets the descriptor bytes each lane reads per poll,
// and so the window: kernels short of registers read narrower windows.
template <typename T, int SPAN, bool STALL, uint32_t SPIN = 0, int LANE_BYTES = 128>
__device__ T lookback(const ScanArgs& a, uint32_t u, uint32_t epoch, uint32_t lane, T carry, int64_t bound,
                      T bound_val) {
    using D = DescTraits<T>;
    using word = typename D::word;
    static_assert(LANE_BYTES >= 16 && LANE_BYTES <= 128 && (LANE_BYTES & (LANE_BYTES - 1)) == 0,
                  "16 to 128 bytes per lane, a power of two");
    constexpr int K = lookback_per_lane<word, LANE_BYTES>();  // slots per lane
    constexpr int PAIR = 16 / static_cast<int>(sizeof(word));  // slots per 16-byte access
    constexpr int NACC = K / PAIR;                      // accesses per lane
    constexpr int WIN = 32 * K;                         // slots per window
    constexpr uint32_t kNone = 0xFFFFFFFFu;
    word* desc = static_cast<word*>(a.desc);
    T prefix = 0;
    int64_t top = (static_cast<int64_t>(u) - 1) | (PAIR - 1);  // top + 1 is a multiple of PAIR
    uint32_t polls = 0;
    uint64_t deadline = 0;
    uint32_t backoff = 64;
    while (true) {
        const int64_t lo = top - WIN + 1;
        // Slot j of this lane: access j / PAIR, element j % PAIR.
        auto slot_idx = [&](int j) -> int64_t {
            return lo + static_cast<int64_t>(j / PAIR) * (32 * PAIR) + lane * PAIR + (j % PAIR);
        };
        T val[K];
        uint32_t valid = 0, incl = 0, pending = 0;
#pragma unroll
        for (int j = 0; j < K; ++j) {
            const int64_t idx = slot_idx(j);
            val[j] = 0;
            if (idx >= static_cast<int64_t>(u)) {
                valid |= 1u << j;  // not a predecessor: an empty aggregate
            } else if (idx <= bound) {
                valid |= 1u << j;  // at or below the bound: an inclusive prefix
                incl |= 1u << j;
                if (idx == bound) val[j] = bound_val;
            } else {
                pending |= 1u << j;  // must be read: (bound, u)
            }
        }
        while (true) {
#pragma unroll
            for (int m = 0; m < NACC; ++m) {
                if ((pending >> (m * PAIR)) & ((1u << PAIR) - 1u)) {
                    const int64_t idx0 = slot_idx(m * PAIR);
                    word wp[PAIR];
                    if constexpr (PAIR == 2) {
                        const ptx::u64x2 r = ptx::ld_relaxed_b128(reinterpret_cast<const ptx::u64x2*>(desc + idx0));
                        wp[0] = r.lo;
                        wp[PAIR - 1] = r.hi;
                    } else {
                        wp[0] = D::load(desc + idx0);
                    }
#pragma unroll
                    for (int q = 0; q < PAIR; ++q) {
                        const int j = m * PAIR + q;
                        if ((pending >> j) & 1u) {
                            const uint32_t st = D::status(wp[q], epoch);
                            if (st != kNotReady) {
                                valid |= 1u << j;
                                pending &= ~(1u << j);
                                val[j] = static_cast<T>(D::value(wp[q]));
                                if (st == kInclusive) incl |= 1u << j;
                            }
                        }
                    }
                }
            }
            // Nearest inclusive position over the warp.
            uint32_t my_incl = kNone;
#pragma unroll
            for (int j = 0; j < K; ++j)
                if ((incl >> j) & 1u) my_incl = min(my_incl, static_cast<uint32_t>(top - slot_idx(j)));
            const uint32_t pinc = __reduce_min_sync(kFullMask, my_incl);
            // Nearest not-ready position nearer than pinc.
            uint32_t my_gap = kNone;
#pragma unroll
            for (int j = 0; j < K; ++j) {
                const uint32_t pos = static_cast<uint32_t>(top - slot_idx(j));
                if (!((valid >> j) & 1u) && pos < pinc) my_gap = min(my_gap, pos);
            }
            const uint32_t gap = __reduce_min_sync(kFullMask, my_gap);
            if (gap == kNone) {
                T part = 0;
#pragma unroll
                for (int j = 0; j < K; ++j)
                    if (static_cast<uint32_t>(top - slot_idx(j)) <= pinc) part += val[j];
                prefix += warp_sum(part);
                if (pinc != kNone) return prefix;
                top -= WIN;  // a window of aggregates only
                polls = 0;
                break;
            }
            // Not resolvable yet: the slot at position `gap` is not ready.
            ++polls;
            if (STALL) {
                if (lane == 0 && a.stall.mode != 0) atomicAdd(&a.hdr->stat_polls, 1ull);
                if (a.stall.fallback_polls != 0 && polls >= a.stall.fallback_polls) {
                    // Re-reduce the nearest predecessor that is still not ready
                    // and try to insert its aggregate.
                    const int64_t fidx = top - gap;
                    const T agg = warp_reduce_tile_input<T, SPAN>(static_cast<const T*>(a.in), a.n,
                                                                 static_cast<uint32_t>(fidx), lane);
                    if (lane == 0) {
                        const word seen = D::load(desc + fidx);
                        if (D::status(seen, epoch) == kNotReady) {
                            __threadfence();
                            const word nw = fidx == 0 ? D::pack(kInclusive, epoch, carry + agg)
                                                      : D::pack(kAggregate, epoch, agg);
                            const word old = D::cas(desc + fidx, seen, nw);
                            atomicAdd(&a.hdr->stat_fallbacks, 1ull);
                            if (D::same(old, seen)) atomicAdd(&a.hdr->stat_inserts, 1ull);
                        }
                    }
                    __syncwarp();
                    polls = 0;
                }
            }
            if ((polls & 15u) == 1u) {
                const uint64_t now = ptx::global_timer_ns();
                if (deadline == 0) deadline = now + a.wait_budget_ns;
                bool give_up = now > deadline || ld_volatile_u32(&a.hdr->error_flags) != 0;
                give_up = __shfl_sync(kFullMask, give_up, 0);
                if (give_up) {
                    if (lane == 0) raise_error(a.hdr, kErrLookbackTimeout);
                    return prefix;
                }
            }
            if (polls > SPIN) {
                __nanosleep(backoff);
                backoff = backoff < 1024 ? backoff * 2 : 1024;
            }
        }
    }
}

// ----------------------------------------------------------- shared state
// Hand-off between the four roles of a CTA, per stage of the ring; each
// mbarrier completes once per use of its stage.
//   full      producer -> reduce    tile landed (bulk-copy bytes) / id set
//   reduced   reduce   -> lookback  aggregate and per-thread offsets ready
//   prefixed  lookback -> finalize  tile prefix ready
//   done      finalize -> producer  scanned tile written back to the stage
template <typename T, int RW, int S>
struct PipeCtrl {
    uint64_t full[S];
    uint64_t reduced[S];
    uint64_t prefixed[S];
    uint64_t done[S];
    uint32_t tile_of[S];
    uint32_t end_iter;  // first iteration without a tile (set by the reduce warps)
    T agg[S];
    T prefix[S];
    T warp_tot[S][RW];
    T offset[S][RW * 32];  // exclusive prefix of each thread's items within the tile
};

template <typename T, int RW, int S>
constexpr size_t pipeline_smem_bytes() {
    return static_cast<size_t>(S) * TileShape<T, RW>::kTile * sizeof(T) + sizeof(PipeCtrl<T, RW, S>);
}

// A 16-byte chunk of elements.
template <typename T>
struct __align__(16) Chunk {
    T v[16 / sizeof(T)];
};

// Logical exclusive prefix of each of the CHUNKS chunks (a power of two) a
// thread holds in rotated order: register j holds chunk (j + rot) % CHUNKS,
// so chunk 0 sits in register (CHUNKS - rot) % CHUNKS. With wrapping integer
// arithmetic the prefix of register j is Q[j] - Q[start], plus the thread
// total when register j comes before start.
template <typename T, int CHUNKS>
__device__ __forceinline__ void rotated_chunk_prefix(const T (&cs)[CHUNKS], uint32_t rot, T (&cpre)[CHUNKS],
                                                     T& total) {
    static_assert(CHUNKS >= 2 && (CHUNKS & (CHUNKS - 1)) == 0, "a power of two of 16-byte chunks per thread");
    T q[CHUNKS];
    T run = 0;
#pragma unroll
    for (int j = 0; j < CHUNKS; ++j) {
        q[j] = run;
        run += cs[j];
    }
    total = run;
    const uint32_t start = (CHUNKS - rot) & (CHUNKS - 1);
    T qstart = 0;
#pragma unroll
    for (int j = 1; j < CHUNKS; ++j) qstart = (static_cast<uint32_t>(j) == start) ? q[j] : qstart;
#pragma unroll
    for (int j = 0; j < CHUNKS; ++j) {
        const bool wraps = rot != 0 && (static_cast<uint32_t>(j) + rot) < static_cast<uint32_t>(CHUNKS);
        cpre[j] = q[j] - qstart + (wraps ? total : T(0));
    }
}

// ------------------------------------------------------------------ kernel
// CTA layout: warp 0 producer, warps 1..LW lookback (taking alternate units),
// then RW reduce warps, then RW finalize warps. Reduce and finalize thread i
// own the same 128 contiguous bytes of a tile, read as eight 16-byte chunks
// in an order rotated by (i & 7) so that each quarter-warp touches all 32
// banks once.
//
// The lookback unit is G consecutive tiles that one CTA loads into G
// consecutive stages: one descriptor and one lookback per unit, so the
// descriptor traffic every CTA reads shrinks G-fold. The ring holds S / G
// units.
//
// Why the roles are split: a unit's aggregate is published as soon as its
// tiles land and are reduced, never behind another unit's lookback, so a
// lookback finds its predecessors' aggregates within about one load latency
// of their ids having been taken. Lookback warps resolve their CTA's units in
// order, so every walk ends at the latest at the unit the same warp (or the
// other lookback warp) resolved before.
template <typename T, int RW, int S, int G, bool INCL, bool BULK, PrefixMode PM, bool STALL>
__global__ void __launch_bounds__(TileShape<T, RW>::kThreads, 2) scan_pipeline_kernel(const ScanArgs a) {
    using Shape = TileShape<T, RW>;
    constexpr int TILE = Shape::kTile;
    constexpr int ITEMS = Shape::kItems;
    constexpr int EPC = 16 / static_cast<int>(sizeof(T));
    constexpr int CHUNKS = ITEMS / EPC;
    constexpr uint32_t NROLE = Shape::kRoleThreads;
    constexpr uint32_t LW = Shape::kLookbackWarps;
    constexpr uint32_t kWarpReduce = 1 + LW, kWarpFinal = 1 + LW + RW;
    constexpr int SLOTS = S / G;
    static_assert(CHUNKS == 8, "128 bytes per thread");
    static_assert(S % G == 0 && SLOTS >= 2, "the ring holds at least two units");
    static_assert(PM == PrefixMode::Lookback || G == 1, "reduce-then-scan works tile by tile");
    using D = DescTraits<T>;
    using word = typename D::word;

    extern __shared__ __align__(1024) uint8_t smem_raw[];
    T* bufs = reinterpret_cast<T*>(smem_raw);
    auto* ctrl = reinterpret_cast<PipeCtrl<T, RW, S>*>(smem_raw + static_cast<size_t>(S) * TILE * sizeof(T));

    const uint32_t tid = threadIdx.x;
    const uint32_t warp = tid >> 5;
    const uint32_t lane = tid & 31u;
    const uint32_t num_units = (a.num_tiles + G - 1) / G;

    if (tid == 0) {
#pragma unroll
        for (int s = 0; s < S; ++s) {
            ptx::mbar_init(&ctrl->full[s], 1);
            ptx::mbar_init(&ctrl->reduced[s], RW);
            ptx::mbar_init(&ctrl->prefixed[s], 1);
            ptx::mbar_init(&ctrl->done[s], RW);
        }
        ctrl->end_iter = 0xFFFFFFFFu;
        ptx::fence_mbar_init();
    }
    __syncthreads();

    const uint32_t epoch = (PM == PrefixMode::Lookback) ? ld_volatile_u32(&a.hdr->epoch) : 0u;
    // Added to every output: the running total of earlier pieces when a long
    // host array is scanned chunk by chunk.
    const T carry = a.carry_in != nullptr ? *static_cast<const T*>(a.carry_in) : T(0);
    const uint64_t budget = a.wait_budget_ns;
    auto count_of = [&](uint32_t t) -> uint32_t {
        return t < a.num_tiles ? tile_count<TILE>(a.n, t) : 0u;
    };
    auto bulk_bytes_of = [&](uint32_t t) -> uint32_t {
        return (count_of(t) * static_cast<uint32_t>(sizeof(T))) & ~15u;
    };

    // ======================================================== producer
    if (warp == 0) {
        if (lane != 0) return;
        bool stop = false;
        uint64_t k_static = 0;
        // Unit ids are taken one refill ahead (acquire) and checked when the
        // refill is issued (resolve), so the counter's round trip overlaps
        // the wait for the finalize warps. Ids only grow, so once one is past
        // the end every later one is too.
        auto acquire = [&]() -> uint64_t {
            if (stop) return ~0ull;
            if (PM == PrefixMode::Spine) return blockIdx.x + (k_static++) * gridDim.x;
            return atomicAdd(&a.hdr->tile_counter, 1u);
        };
        auto resolve = [&](uint64_t raw) -> uint32_t {
            if (stop || raw >= num_units ||
                (PM == PrefixMode::Lookback && ld_volatile_u32(&a.hdr->error_flags) != 0)) {
                stop = true;
                return kTileEnd;
            }
            return static_cast<uint32_t>(raw);
        };
        auto issue = [&](int j, uint32_t u) {
#pragma unroll 1
            for (int k = 0; k < G; ++k) {
                const int s = j * G + k;
                const uint32_t t = u == kTileEnd ? kTileEnd : u * G + k;
                ctrl->tile_of[s] = t;
                if (BULK && t != kTileEnd) {
                    const uint32_t bytes = bulk_bytes_of(t);
                    ptx::mbar_arrive_expect_tx(&ctrl->full[s], bytes);
                    if (bytes)
                        ptx::bulk_load(bufs + static_cast<size_t>(s) * TILE,
                                       static_cast<const T*>(a.in) + static_cast<uint64_t>(t) * TILE, bytes,
                                       &ctrl->full[s]);
                } else {
                    ptx::mbar_arrive(&ctrl->full[s]);
                }
            }
        };
#pragma unroll 1
        for (int j = 0; j < SLOTS; ++j) issue(j, resolve(acquire()));
        uint64_t upcoming = acquire();

        const uint64_t long_budget = budget * 4 + 1000000000ull;
        bool failed = false;
        for (uint32_t i = 0; !failed; ++i) {
            const int j = static_cast<int>(i % SLOTS);
            const uint32_t ph = (i / SLOTS) & 1u;
            if (ctrl->tile_of[j * G] == kTileEnd) break;
#pragma unroll 1
            for (int k = 0; k < G; ++k) {
                const int s = j * G + k;
                if (!ptx::mbar_try_wait(&ctrl->done[s], ph) &&
                    !ptx::mbar_wait_bounded(&ctrl->done[s], ph, ptx::global_timer_ns() + long_budget)) {
                    raise_error(a.hdr, kErrPipelineTimeout);
                    failed = true;
                    break;
                }
                if (BULK) {
                    const uint32_t t = ctrl->tile_of[s];
                    const uint32_t bytes = t == kTileEnd ? 0u : bulk_bytes_of(t);
                    if (bytes)
                        ptx::bulk_store(static_cast<T*>(a.out) + static_cast<uint64_t>(t) * TILE,
                                        bufs + static_cast<size_t>(s) * TILE, bytes);
                }
            }
            if (failed) break;
            // Refill the slot as soon as its stores have read it out.
            if (BULK) {
                ptx::bulk_commit();
                ptx::bulk_wait_read<0>();
            }
            issue(j, resolve(upcoming));
            upcoming = acquire();
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
                    for (unsigned long long q = 0; q < a.hdr->capacity_tiles; ++q) D::store(desc + q, D::zero());
                    e += 1;
                }
                __threadfence();
                a.hdr->epoch = e;
            }
        }
        return;
    }

    // ======================================================== lookback
    if (warp <= LW) {
        word* desc = static_cast<word*>(a.desc);
        // Inclusive prefix through the last unit this warp resolved: every
        // later walk of this warp stops there at the latest.
        int64_t own_prev = -1;
        T own_incl = 0;
        // Lane 0 waits on a stage barrier; while waiting it also watches
        // end_iter, the first unit the reduce warps did not take.
        // Returns 0 (phase complete), 1 (no such unit) or 2 (wait ran out).
        auto wait_stage = [&](uint64_t* bar, uint32_t ph, uint32_t i, uint64_t wait_budget) -> uint32_t {
            uint32_t state = 0;
            if (lane == 0) {
                uint64_t deadline = 0;
                uint32_t polls = 0;
                while (!ptx::mbar_try_wait(bar, ph)) {
                    if (ld_volatile_u32(&ctrl->end_iter) <= i) {
                        state = 1;
                        break;
                    }
                    if ((++polls & 63u) == 0) {
                        const uint64_t now = ptx::global_timer_ns();
                        if (deadline == 0) {
                            deadline = now + wait_budget;
                        } else if (now > deadline) {
                            state = 2;
                            break;
                        }
                    }
                }
            }
            __syncwarp();
            return __shfl_sync(kFullMask, state, 0);
        };
        for (uint32_t i = warp - 1;; i += LW) {
            const int j = static_cast<int>(i % SLOTS);
            const uint32_t ph = (i / SLOTS) & 1u;
            // The unit id is known once its first tile has landed; the walk
            // over the predecessors' descriptors starts right away, while the
            // reduce warps are still summing this unit's tiles.
            uint32_t state = wait_stage(&ctrl->full[j * G], ph, i, budget * 2);
            const uint32_t t0 = state == 0 ? ctrl->tile_of[j * G] : kTileEnd;
            if (state == 2 || t0 == kTileEnd) {
                if (lane == 0) {
                    if (state == 2) raise_error(a.hdr, kErrPipelineTimeout);
                    // The finalize warps stop at the first stage without a tile.
                    if (state == 0) ptx::mbar_arrive(&ctrl->prefixed[j * G]);
                }
                break;
            }
            const uint32_t u = t0 / G;
            T pre;
            if (PM == PrefixMode::Spine) {
                pre = carry + (t0 == 0 ? T(0) : static_cast<const T*>(a.spine)[t0 - 1]);
            } else if (u == 0) {
                pre = carry;
            } else {
                int64_t bound = own_prev;
                T bound_val = own_incl;
                if (LW > 1 && i >= 1) {
                    // The other lookback warp's unit of the previous iteration
                    // is nearer; use it if it is already resolved.
                    const int j1 = static_cast<int>((i - 1) % SLOTS);
                    const int s1 = j1 * G + G - 1;
                    const bool r1 =
                        __all_sync(kFullMask, ptx::mbar_test_wait(&ctrl->prefixed[s1], ((i - 1) / SLOTS) & 1u));
                    if (r1) {
                        const uint32_t u1 = ctrl->tile_of[j1 * G] / G;
                        if (static_cast<int64_t>(u1) > bound && u1 < u) {
                            bound = u1;
                            bound_val = ctrl->prefix[s1] + ctrl->agg[s1];
                        }
                    }
                }
                pre = lookback<T, TILE * G, STALL>(a, u, epoch, lane, carry, bound, bound_val);
            }
            // Hand each tile its prefix as soon as its own aggregate is in.
            T run = pre;
            bool stopped = false;
#pragma unroll 1
            for (int k = 0; k < G; ++k) {
                const int s = j * G + k;
                state = wait_stage(&ctrl->reduced[s], ph, i, budget * 2);
                if (state != 0) {
                    if (lane == 0 && state == 2) raise_error(a.hdr, kErrPipelineTimeout);
                    stopped = true;
                    break;
                }
                if (lane == 0) {
                    ctrl->prefix[s] = run;
                    if (STALL && k == G - 1) __threadfence();
                    ptx::mbar_arrive(&ctrl->prefixed[s]);
                }
                run += ctrl->agg[s];
            }
            if (stopped) break;
            if (PM == PrefixMode::Lookback && u != 0 && lane == 0) D::store(desc + u, D::pack(kInclusive, epoch, run));
            if (lane == 0 && a.carry_out != nullptr && u == num_units - 1) *static_cast<T*>(a.carry_out) = run;
            own_prev = u;
            own_incl = run;
            __syncwarp();
        }
        return;
    }

    // ======================================================== reduce
    if (warp < kWarpFinal) {
        const uint32_t r = tid - kWarpReduce * 32;
        const uint32_t rw = warp - kWarpReduce;
        const uint32_t rot = r & 7u;
        bool running = true;
        for (uint32_t i = 0; running; ++i) {
            const int j = static_cast<int>(i % SLOTS);
            const uint32_t ph = (i / SLOTS) & 1u;
            T unit_agg = 0;
#pragma unroll 1
            for (int k = 0; k < G; ++k) {
                const int s = j * G + k;
                const bool ok = ptx::mbar_try_wait(&ctrl->full[s], ph) ||
                                ptx::mbar_wait_bounded(&ctrl->full[s], ph, ptx::global_timer_ns() + budget);
                const uint32_t t = ok ? ctrl->tile_of[s] : kTileEnd;
                const bool live = t != kTileEnd;
                T* sb = bufs + static_cast<size_t>(s) * TILE;
                const uint32_t cnt = live ? count_of(t) : 0u;
                T total = 0;
                if (BULK && cnt == static_cast<uint32_t>(TILE)) {
#pragma unroll
                    for (int c8 = 0; c8 < CHUNKS; ++c8) {
                        const uint32_t c = (c8 + rot) & (CHUNKS - 1);
                        const Chunk<T> q = *reinterpret_cast<const Chunk<T>*>(sb + r * ITEMS + c * EPC);
#pragma unroll
                        for (int e = 0; e < EPC; ++e) total += q.v[e];
                    }
                } else if (cnt != 0) {
                    // Partial tile or unaligned buffers: elements the bulk copy
                    // did not bring in are read from global memory and parked
                    // in the stage, so that finalize always reads the stage.
                    const uint32_t bulk_elems = BULK ? bulk_bytes_of(t) / static_cast<uint32_t>(sizeof(T)) : 0u;
                    const uint64_t gbase = static_cast<uint64_t>(t) * TILE;
#pragma unroll 4
                    for (int e = 0; e < ITEMS; ++e) {
                        const uint32_t li = r * ITEMS + e;
                        T x = 0;
                        if (li < cnt) {
                            if (BULK && li < bulk_elems) {
                                x = sb[li];
                            } else {
                                x = static_cast<const T*>(a.in)[gbase + li];
                                sb[li] = x;
                            }
                        }
                        total += x;
                    }
                }
                const T winc = warp_inclusive_scan(total, lane);
                if (lane == 31) ctrl->warp_tot[s][rw] = winc;
                // Agree on "stop" (end of units, or a wait that ran out).
                if (named_bar_or(1, NROLE, !live)) {
                    if (r == 0) {
                        if (!ok) {
                            raise_error(a.hdr, kErrPipelineTimeout);
                            ctrl->tile_of[s] = kTileEnd;
                        }
                        *reinterpret_cast<volatile uint32_t*>(&ctrl->end_iter) = i;
                    }
                    __syncwarp();
                    if (lane == 0) ptx::mbar_arrive(&ctrl->reduced[s]);
                    running = false;
                    break;
                }
                T wpre = 0, agg = 0;
#pragma unroll
                for (int w2 = 0; w2 < RW; ++w2) {
                    const T x = ctrl->warp_tot[s][w2];
                    wpre += (static_cast<uint32_t>(w2) < rw) ? x : T(0);
                    agg += x;
                }
                ctrl->offset[s][r] = wpre + winc - total;
                if (r == 0) {
                    ctrl->agg[s] = agg;
                    unit_agg += agg;
                    if (PM == PrefixMode::Lookback && k == G - 1) {
                        const uint32_t u = t / G;
                        word* desc = static_cast<word*>(a.desc);
                        bool publish = true;
                        if (STALL && unit_stalls(a.stall, u, (a.num_tiles + G - 1) / G)) {
                            // Withhold the aggregate until the delay ends or a
                            // successor inserts it (EmulatedDeadlocking.cuh:64-70).
                            atomicAdd(&a.hdr->stat_stalls, 1ull);
                            const uint64_t until = ptx::global_timer_ns() + a.stall.delay_ns;
                            while (true) {
                                if (D::status(D::load(desc + u), epoch) != kNotReady) {
                                    publish = false;
                                    break;
                                }
                                if (ptx::global_timer_ns() > until) break;
                                __nanosleep(200);
                            }
                        }
                        // Only unit 0's value is an inclusive prefix, so only
                        // it holds the carry. A rescuer computes the same
                        // integer aggregate, so a plain store over an inserted
                        // one is harmless; rescuers use a CAS so that they
                        // never overwrite an inclusive prefix.
                        if (publish)
                            D::store(desc + u, u == 0 ? D::pack(kInclusive, epoch, carry + unit_agg)
                                                      : D::pack(kAggregate, epoch, unit_agg));
                    }
                }
                __syncwarp();
                if (lane == 0) ptx::mbar_arrive(&ctrl->reduced[s]);
            }
        }
        return;
    }

    // ======================================================== finalize
    {
        const uint32_t f = tid - kWarpFinal * 32;
        const uint32_t rot = f & 7u;
        bool running = true;
        for (uint32_t i = 0; running; ++i) {
            const int j = static_cast<int>(i % SLOTS);
            const uint32_t ph = (i / SLOTS) & 1u;
#pragma unroll 1
            for (int k = 0; k < G; ++k) {
                const int s = j * G + k;
                bool ok = ptx::mbar_try_wait(&ctrl->prefixed[s], ph) ||
                          ptx::mbar_wait_bounded(&ctrl->prefixed[s], ph, ptx::global_timer_ns() + budget * 3);
                ok = __all_sync(kFullMask, ok);
                const uint32_t t = ok ? ctrl->tile_of[s] : kTileEnd;
                if (t == kTileEnd) {
                    if (!ok && lane == 0) raise_error(a.hdr, kErrPipelineTimeout);
                    running = false;
                    break;
                }
                T* sb = bufs + static_cast<size_t>(s) * TILE;
                const uint32_t cnt = count_of(t);
                const T base = ctrl->prefix[s] + ctrl->offset[s][f];
                if (BULK && cnt == static_cast<uint32_t>(TILE)) {
                    T v[ITEMS];
                    T cs[CHUNKS];
#pragma unroll
                    for (int c8 = 0; c8 < CHUNKS; ++c8) {
                        const uint32_t c = (c8 + rot) & (CHUNKS - 1);
                        const Chunk<T> q = *reinterpret_cast<const Chunk<T>*>(sb + f * ITEMS + c * EPC);
                        T x = 0;
#pragma unroll
                        for (int e = 0; e < EPC; ++e) {
                            v[c8 * EPC + e] = q.v[e];
                            x += q.v[e];
                        }
                        cs[c8] = x;
                    }
                    T cpre[CHUNKS];
                    T total;
                    rotated_chunk_prefix<T, CHUNKS>(cs, rot, cpre, total);
#pragma unroll
                    for (int c8 = 0; c8 < CHUNKS; ++c8) {
                        T run = base + cpre[c8];
                        Chunk<T> q;
#pragma unroll
                        for (int e = 0; e < EPC; ++e) {
                            const T x = v[c8 * EPC + e];
                            if (INCL) {
                                run += x;
                                q.v[e] = run;
                            } else {
                                q.v[e] = run;
                                run += x;
                            }
                        }
                        const uint32_t c = (c8 + rot) & (CHUNKS - 1);
                        *reinterpret_cast<Chunk<T>*>(sb + f * ITEMS + c * EPC) = q;
                    }
                } else if (cnt != 0) {
                    const uint32_t bulk_elems = BULK ? bulk_bytes_of(t) / static_cast<uint32_t>(sizeof(T)) : 0u;
                    const uint64_t gbase = static_cast<uint64_t>(t) * TILE;
                    T run = base;
#pragma unroll 4
                    for (int e = 0; e < ITEMS; ++e) {
                        const uint32_t li = f * ITEMS + e;
                        if (li < cnt) {
                            const T x = sb[li];
                            const T y = INCL ? run + x : run;
                            run += x;
                            if (BULK && li < bulk_elems)
                                sb[li] = y;
                            else
                                static_cast<T*>(a.out)[gbase + li] = y;
                        }
                    }
                }
                if (BULK) ptx::fence_proxy_async_smem();
                __syncwarp();
                if (lane == 0) ptx::mbar_arrive(&ctrl->done[s]);
            }
        }
    }
}

}  // namespace gps
