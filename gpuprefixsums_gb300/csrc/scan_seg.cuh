// Generic single-pass scan, L2-buffered like scan_l2.cuh, over any scan
// operation of scan_ops.cuh, optionally segmented (batched).
//
// Batched / segmented mode: thousands of independent scans packed one after
// the other and described by CSR offsets (segment s is
// [offsets[s], offsets[s+1])) run as ONE launch at streaming bandwidth. Each
// element carries a "segment head" bit; states combine with the segmented
// operator
//     (a, fa) . (b, fb) = (fb ? b : a + b, fa | fb),
// which is associative, so the same decoupled lookback works: a unit whose
// tiles contain a head publishes the sum since its last head together with a
// head flag, and such a descriptor ends a lookback walk just like an
// inclusive prefix. Short segments therefore resolve inside their unit, long
// ones walk back to the unit where they start. The reference has no batched
// or floating-point scan; this kernel covers those rows of the design
// (dtype per launch: u32, u64, plain FP32, compensated FP32, and structs of
// four u32 members).
//
// Warps: 0 R-loader, 1 S-loader, 2 storer, 3 head warp (segment heads of each
// unit, from the offsets), then LW lookback warps, the aggregator warp, RW
// reduce warps and RW finalize warps; see scan_l2.cuh for the two passes.
// Unlike scan_l2.cuh, the reduce warps only aggregate their rows: once per
// unit the aggregator warp scans those aggregates, publishes the unit's
// aggregate and hands every finalize thread its state within the unit, so
// neither pass has a warp scan or a barrier per tile.
#pragma once
#include <type_traits>

#include "scan_ops.cuh"
#include "scan_pipeline.cuh"

namespace gps {

// 128-bit descriptor of the generic kernel:
//   lo: chain value bits; hi: status:2 (bits 63-62) | head flag (bit 61) |
//   epoch:30 (bits 29-0). Same status/epoch placement as the u64 descriptor.
constexpr uint64_t kHeadFlagBit = 1ull << 61;

__device__ __forceinline__ ptx::u64x2 seg_pack(uint32_t status, bool flag, uint32_t epoch, uint64_t bits) {
    ptx::u64x2 w;
    w.lo = bits;
    w.hi = (static_cast<uint64_t>(status) << 62) | (flag ? kHeadFlagBit : 0ull) | (epoch & kEpochMask);
    return w;
}

// Segmented combine of (a, fa) followed by (b, fb).
template <class Op>
__device__ __forceinline__ void seg_combine(typename Op::S& a, bool& fa, typename Op::S b, bool fb) {
    a = fb ? b : Op::combine(a, b);
    fa = fa || fb;
}

template <class Op>
__device__ __forceinline__ typename Op::C chain_warp_sum(typename Op::C x) {
#pragma unroll
    for (int m = 16; m; m >>= 1) x = Op::chain_add(x, Op::chain_shfl_xor(x, m));
    return x;
}

// Inclusive warp scan of (state, head flag) in lane order. Without FLAGS the
// flags are known to be false and only the states move.
template <class Op, bool FLAGS>
__device__ __forceinline__ void warp_scan_incl(typename Op::S& s, bool& f, uint32_t lane) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const typename Op::S ov = Op::shfl_up(s, d);
        const bool of = FLAGS ? __shfl_up_sync(kFullMask, f, d) : false;
        if (lane >= static_cast<uint32_t>(d)) {
            if (FLAGS) {
                s = f ? s : Op::combine(ov, s);
                f = f || of;
            } else {
                s = Op::combine(ov, s);
            }
        }
    }
}

// Aggregate of a thread's items in logical order; hb holds their head bits
// (HEADS = false: no item of the warp is a segment head). One chain, whose
// step is one add (one FP32 add on hi and one on lo for the compensated
// scan, see scan_ops.cuh).
template <class Op, int ITEMS, bool HEADS>
__device__ __forceinline__ typename Op::S thread_aggregate(const typename Op::T (&v)[ITEMS], uint32_t hb) {
    if constexpr (!HEADS && Op::kPackedRowSum) return Op::template row_sum<ITEMS>(v);
    typename Op::S x = Op::zero();
#pragma unroll
    for (int e = 0; e < ITEMS; ++e) x = (HEADS && ((hb >> e) & 1u)) ? Op::lift(v[e]) : Op::acc(x, v[e]);
    return Op::norm(x);
}

// Scanned outputs of a thread's items from the state before its first item.
template <class Op, int ITEMS, bool HEADS, bool INCL>
__device__ __forceinline__ void thread_outputs(typename Op::T (&v)[ITEMS], typename Op::S st, uint32_t hb) {
#pragma unroll
    for (int e = 0; e < ITEMS; ++e) {
        const typename Op::S before = (HEADS && ((hb >> e) & 1u)) ? Op::zero() : st;
        st = Op::acc(before, v[e]);
        v[e] = INCL ? Op::out(st) : Op::out(before);
    }
}

// Words from one unit descriptor (or group descriptor) to the next.
template <class Op>
__device__ __forceinline__ uint32_t desc_words(const ScanArgs& a) {
    return a.desc_stride != 0 ? a.desc_stride : static_cast<uint32_t>(Op::kDescWords);
}

// A unit's descriptor is Op::kDescWords 128-bit words, each carrying one
// 64-bit word of the chain value with the status, head flag and epoch: a
// reader takes the value only when every word has the launch's epoch and
// the same status (a word that is one publication behind reads as not
// ready). Descriptor u starts at word u * ws: ws is Op::kDescWords (packed)
// or a.desc_stride (one 128-byte line per descriptor, see desc_words()).
template <class Op>
__device__ __forceinline__ void desc_store(ptx::u64x2* desc, uint64_t u, uint32_t ws, uint32_t status, bool flag,
                                           uint32_t epoch, typename Op::C c) {
#pragma unroll
    for (int w = 0; w < Op::kDescWords; ++w)
        ptx::st_relaxed_b128(desc + u * ws + w, seg_pack(status, flag, epoch, Op::chain_word(c, w)));
}

template <class Op>
__device__ __forceinline__ uint32_t desc_load(const ptx::u64x2* desc, uint64_t u, uint32_t ws, uint32_t epoch,
                                              bool& flag, typename Op::C& c) {
    uint64_t words[Op::kDescWords];
    uint32_t st = kNotReady;
#pragma unroll
    for (int w = 0; w < Op::kDescWords; ++w) {
        const ptx::u64x2 x = ptx::ld_relaxed_b128(desc + u * ws + w);
        const uint32_t s = (static_cast<uint32_t>(x.hi) & kEpochMask) == (epoch & kEpochMask)
                               ? static_cast<uint32_t>(x.hi >> 62)
                               : kNotReady;
        if (w == 0) {
            st = s;
            flag = (x.hi & kHeadFlagBit) != 0;
        } else if (s != st) {
            st = kNotReady;
        }
        words[w] = x.lo;
    }
    if (st != kNotReady) c = Op::chain_from_words(words);
    return st;
}

// Lookback of the generic kernel, in a fixed order. A decoupled lookback
// that sums whichever predecessors' descriptors it finds ready makes the
// rounding of a floating-point prefix depend on timing; here the units form
// groups of G = kDetGroupUnits, a unit's descriptor holds its aggregate only
// (it is never upgraded to an inclusive prefix), and the prefix of unit u in
// group g is
//     P(g) + fold(aggregates of units G*g .. u-1),
// where the fold has a fixed shape (each lane folds its G/32 consecutive
// units in order, then an order-keeping butterfly over the lanes) and P(g),
// the prefix before group g, is a chain: the last unit of each group
// publishes P(g + 1) = prefix + aggregate in the group descriptor array, as
// an inclusive value. Every addition has fixed operands in a fixed order, so
// a launch configuration gives bitwise-identical results from run to run.
// Segment heads fold in the same order, and a head among the in-group
// predecessors makes P(g) unnecessary. The group prefixes pass from group to
// group one at a time, one L2 round trip per G units, which stays off the
// critical path while G units take longer to stream than that round trip.
// Measured on GB300 against the lookback that stops at the nearest
// inclusive prefix (windows of 256 descriptors, back-off up to 1 us): 2^28
// FP32 in 333 against 342 us, compensated 344 against 355 us, 4096 batched
// u32 segments (305 M elements) in 381 against 395 us, compensated FP32
// 506 against 564 us (units of 4 tiles). Groups of 256 units took 348, 357,
// 390 and 502 us. A back-off of up to 1 us instead of 128 ns while waiting
// took 338, 349, 380 and 502 us, and 656 against 555 us for 2^28 FP32 in
// single-tile units, where a group streams in about a microsecond.
static_assert(kDetGroupUnits % 32 == 0 && kDetGroupUnits <= 32 * 32, "whole lanes of at most 32 units");

template <class Op>
__device__ typename Op::C seg_lookback(const ScanArgs& a, uint32_t u, uint32_t epoch, uint32_t lane) {
    using C = typename Op::C;
    const uint32_t ws = desc_words<Op>(a);
    constexpr int K = static_cast<int>(kDetGroupUnits / 32);  // units per lane
    const ptx::u64x2* desc = static_cast<const ptx::u64x2*>(a.desc);
    const ptx::u64x2* gdesc = static_cast<const ptx::u64x2*>(a.group_desc);
    const uint32_t g = u / kDetGroupUnits;
    const uint32_t i0 = g * kDetGroupUnits;
    const uint32_t cnt = u - i0;  // in-group predecessors
    C v[K];
    bool f[K];
    uint32_t ready = 0;
#pragma unroll
    for (int j = 0; j < K; ++j) {
        v[j] = Op::chain_zero();
        f[j] = false;
        if (lane * K + j >= cnt) ready |= 1u << j;  // not a predecessor: identity
    }
    uint32_t polls = 0, backoff = 64;
    uint64_t deadline = 0;
    auto expired = [&]() -> bool {
        ++polls;
        if ((polls & 15u) == 1u) {
            const uint64_t now = ptx::global_timer_ns();
            if (deadline == 0) deadline = now + a.wait_budget_ns;
            bool give_up = now > deadline || ld_volatile_u32(&a.hdr->error_flags) != 0;
            give_up = __shfl_sync(kFullMask, give_up, 0);
            if (give_up) {
                if (lane == 0) raise_error(a.hdr, kErrLookbackTimeout);
                return true;
            }
        }
        __nanosleep(backoff);
        backoff = backoff < 128 ? backoff * 2 : 128;
        return false;
    };
    // 1. The in-group aggregates.
    while (true) {
#pragma unroll
        for (int j = 0; j < K; ++j) {
            if (!((ready >> j) & 1u)) {
                bool hf = false;
                C cv;
                if (desc_load<Op>(desc, i0 + lane * K + j, ws, epoch, hf, cv) != kNotReady) {
                    v[j] = cv;
                    f[j] = hf;
                    ready |= 1u << j;
                }
            }
        }
        if (__all_sync(kFullMask, ready == (1u << K) - 1u)) break;
        if (expired()) return Op::chain_zero();
    }
    // 2. Their fold in a fixed shape, in unit order.
    C c = v[0];
    bool fl = f[0];
#pragma unroll
    for (int j = 1; j < K; ++j) {
        c = f[j] ? v[j] : Op::chain_add(c, v[j]);
        fl = fl || f[j];
    }
#pragma unroll
    for (int m = 1; m < 32; m <<= 1) {
        const C oc = Op::chain_shfl_xor(c, m);
        const bool of = __shfl_xor_sync(kFullMask, fl, m) != 0;
        if (lane & static_cast<uint32_t>(m))
            c = fl ? c : Op::chain_add(oc, c);  // the partner holds the block on the left
        else
            c = of ? oc : Op::chain_add(c, oc);
        fl = fl || of;
    }
    if (fl || g == 0) return c;
    // 3. The group prefix (every lane reads the one descriptor; it is
    // written once per launch, so all lanes that see it see the same value).
    C gp = Op::chain_zero();
    while (true) {
        bool hf = false;
        const bool ok = desc_load<Op>(gdesc, g - 1, ws, epoch, hf, gp) == kInclusive;
        if (__all_sync(kFullMask, ok)) break;
        if (expired()) return Op::chain_zero();
    }
    return Op::chain_add(gp, c);
}

template <class Op, int RW, int RS, int SS, int Q, int G, bool SEG>
struct SegCtrl {
    using S = typename Op::S;
    using C = typename Op::C;
    static constexpr int kHeadWords = 16384 / static_cast<int>(sizeof(typename Op::T)) / 32;
    uint64_t rfull[RS], rfree[RS];
    uint64_t sfull[SS], sdone[SS], sfree[SS];
    uint64_t uknown[Q], uheads[Q], uentries[Q], ureduced[Q], ustates[Q], uprefix[Q], ufree[Q];
    uint32_t r_tile[RS];
    uint32_t s_tile[SS];
    uint32_t unit_of[Q];
    uint32_t end_seq;
    uint32_t uflag[Q];  // unit holds a segment head
    C uagg[Q];
    C upre[Q];
    // Per unit, one entry per reduce thread and tile (E = G * RW * 32, in
    // unit order): the reduce warps leave each thread's aggregate there, the
    // aggregator warp replaces it by the state before that thread within the
    // unit, which the scan pass reads. Entry j sits at j + j / (G * RW), so
    // that the aggregator's lanes, which take G * RW consecutive entries
    // each, and the threads of a warp, which take consecutive ones, both
    // meet distinct banks.
    static constexpr int kEntries = G * RW * 32;
    S tpre[Q][kEntries + 32];
    // Segmented scans: per entry, first "the thread's items hold a head",
    // then "a head lies between the unit's start and the thread".
    uint8_t tflag[SEG ? Q : 1][SEG ? kEntries : 1];
    // Segmented scans only (one unused entry otherwise):
    uint32_t heads[SEG ? Q : 1][G][kHeadWords];  // bit b of word w: element 32w+b is a segment head
    uint32_t sample[SEG ? 1024 : 1];             // offsets[j * sample_stride], to start head searches
};

template <class Op, int RW, int RS, int SS, int Q, int G, bool SEG>
constexpr size_t seg_smem_bytes() {
    return static_cast<size_t>(RS + SS) * 16384 +
           sizeof(SegCtrl<Op, RW, RS, SS, Q, G, SEG>);
}

template <class Op, int RW>
struct SegShape {
    static constexpr int kLookbackWarps = 3;
    // R-loader, S-loader, storer, head warp, lookback warps, aggregator,
    // reduce warps, finalize warps.
    static constexpr int kThreads = 32 * (5 + kLookbackWarps + 2 * RW);
};

template <class Op, int RW, int RS, int SS, int Q, int G, bool INCL, bool SEG>
__global__ void __launch_bounds__(SegShape<Op, RW>::kThreads, 1)
    scan_seg_kernel(const ScanArgs a, const SegArgs sg, const __grid_constant__ CUtensorMap tin,
                    const __grid_constant__ CUtensorMap tout) {
    using T = typename Op::T;
    using S = typename Op::S;
    using C = typename Op::C;
    // A tile is 128 rows of 128 bytes (16 KB). Each role has RW warps:
    // SPLIT = RW / 4 threads share a row (1 or 2), so a thread holds
    // 128 / SPLIT bytes: ITEMS elements in CHUNKS 16-byte chunks.
    constexpr int SPLIT = RW / 4;
    constexpr int TILE = 16384 / static_cast<int>(sizeof(T));
    constexpr int ITEMS = 128 / static_cast<int>(sizeof(T)) / SPLIT;
    constexpr int EPC = 16 / static_cast<int>(sizeof(T));
    constexpr int CHUNKS = ITEMS / EPC;
    constexpr uint32_t NROLE = RW * 32;
    constexpr uint32_t ROWS = 128;  // rows per tile
    constexpr uint32_t LW = SegShape<Op, RW>::kLookbackWarps;
    constexpr uint32_t kWarpLookback = 4, kWarpAgg = 4 + LW, kWarpReduce = 5 + LW, kWarpFinal = 5 + LW + RW;
    constexpr uint32_t kLaneEntries = G * RW;  // aggregator entries per lane
    auto entry_at = [](uint32_t j) -> uint32_t { return j + j / kLaneEntries; };
    constexpr int kHeadWords = TILE / 32;
    static_assert((SPLIT == 1 || SPLIT == 2) && RW % 4 == 0, "4 or 8 warps per role");
    static_assert(NROLE / SPLIT == ROWS, "a tile is one box of 128 rows of 128 bytes");
    static_assert(Q > LW, "every lookback warp needs its own queue entry");
    using Ctrl = SegCtrl<Op, RW, RS, SS, Q, G, SEG>;

    extern __shared__ __align__(1024) uint8_t smem_raw[];
    T* rbuf = reinterpret_cast<T*>(smem_raw);
    T* sbuf = rbuf + static_cast<size_t>(RS) * TILE;
    Ctrl* ctrl = reinterpret_cast<Ctrl*>(smem_raw + static_cast<size_t>(RS + SS) * TILE * sizeof(T));

    const uint32_t tid = threadIdx.x;
    const uint32_t warp = tid >> 5;
    const uint32_t lane = tid & 31u;
    const uint32_t num_units = (a.num_tiles + G - 1) / G;
    // The 128-byte swizzle repeats every 1024 bytes: stages must start on a
    // 1024-byte boundary. (A misaligned window is reported, not used.)
    if ((ptx::smem_addr(smem_raw) & 1023u) != 0) {
        if (tid == 0) raise_error(a.hdr, kErrPipelineTimeout);
        return;
    }
    // Rows of 128 bytes: full ones move by TMA; the last, partial row (the
    // n % ROW tail) by plain loads and stores of its owning thread.
    constexpr uint32_t ROW = 128 / sizeof(T);
    const uint64_t rows_full = a.n / ROW;
    const uint32_t tail = static_cast<uint32_t>(a.n % ROW);
    // Samples of the offsets: every `stride`-th entry, at most 1024.
    const uint32_t nseg = SEG ? sg.num_segments : 0u;
    const uint32_t stride = SEG ? (nseg + 1 + 1023) / 1024 : 1u;
    const uint32_t nsample = SEG ? (nseg + stride) / stride : 0u;  // samples cover entries 0..nseg

    if (tid == 0) {
        for (int s = 0; s < RS; ++s) {
            ptx::mbar_init(&ctrl->rfull[s], 1);
            ptx::mbar_init(&ctrl->rfree[s], RW);
        }
        for (int s = 0; s < SS; ++s) {
            ptx::mbar_init(&ctrl->sfull[s], 1);
            ptx::mbar_init(&ctrl->sdone[s], RW);
            ptx::mbar_init(&ctrl->sfree[s], 1);
        }
        for (int q = 0; q < Q; ++q) {
            ptx::mbar_init(&ctrl->uknown[q], 1);
            ptx::mbar_init(&ctrl->uheads[q], 1);
            ptx::mbar_init(&ctrl->uentries[q], RW);
            ptx::mbar_init(&ctrl->ustates[q], 1);
            ptx::mbar_init(&ctrl->ureduced[q], 1);
            ptx::mbar_init(&ctrl->uprefix[q], 1);
            ptx::mbar_init(&ctrl->ufree[q], RW);
        }
        ctrl->end_seq = 0xFFFFFFFFu;
        ptx::fence_mbar_init();
    }
    if constexpr (SEG)
        for (uint32_t j = tid; j < nsample; j += blockDim.x) ctrl->sample[j] = sg.offsets[min(j * stride, nseg)];
    __syncthreads();

    const uint32_t epoch = ld_volatile_u32(&a.hdr->epoch);
    const uint64_t budget = a.wait_budget_ns;
    const uint64_t long_budget = budget * 4 + 1000000000ull;
    // Bytes one TMA box brings for tile t (rows past the tensor are filled
    // with zeros and counted), or 0 when the tile has no full row.
    auto tma_bytes_of = [&](uint32_t t) -> uint32_t {
        return (t < a.num_tiles && static_cast<uint64_t>(t) * ROWS < rows_full)
                   ? static_cast<uint32_t>(TILE * sizeof(T))
                   : 0u;
    };
    // A thread's part of its 128-byte row of tile t (all of it, or one of
    // two halves), in logical order. In the stage, chunk j of row r sits at
    // j ^ (r & 7) (the 128-byte swizzle): 8 consecutive threads touch 8
    // different 16-byte bank groups.
    auto load_row = [&](const T* stage, uint32_t t, uint32_t thr, T (&v)[ITEMS]) {
        const uint32_t rit = thr / SPLIT, sub = thr % SPLIT;
        const uint64_t row = static_cast<uint64_t>(t) * ROWS + rit;
        if (row < rows_full) {
            const T* rp = stage + rit * ROW;
#pragma unroll
            for (int c = 0; c < CHUNKS; ++c) {
                const int pos = (static_cast<int>(sub) * CHUNKS + c) ^ static_cast<int>(rit & 7u);
                const Chunk<T> qv = *reinterpret_cast<const Chunk<T>*>(rp + pos * EPC);
#pragma unroll
                for (int e = 0; e < EPC; ++e) v[c * EPC + e] = qv.v[e];
            }
        } else {
            const T* gp = static_cast<const T*>(a.in) + row * ROW + sub * ITEMS;
#pragma unroll
            for (int e = 0; e < ITEMS; ++e)
                v[e] = (row == rows_full && sub * ITEMS + static_cast<uint32_t>(e) < tail) ? gp[e] : T{};
        }
    };
    auto store_row = [&](T* stage, uint32_t t, uint32_t thr, const T (&v)[ITEMS]) {
        const uint32_t rit = thr / SPLIT, sub = thr % SPLIT;
        const uint64_t row = static_cast<uint64_t>(t) * ROWS + rit;
        if (row < rows_full) {
            T* rp = stage + rit * ROW;
#pragma unroll
            for (int c = 0; c < CHUNKS; ++c) {
                Chunk<T> qv;
#pragma unroll
                for (int e = 0; e < EPC; ++e) qv.v[e] = v[c * EPC + e];
                const int pos = (static_cast<int>(sub) * CHUNKS + c) ^ static_cast<int>(rit & 7u);
                *reinterpret_cast<Chunk<T>*>(rp + pos * EPC) = qv;
            }
        } else if (row == rows_full) {
            T* gp = static_cast<T*>(a.out) + row * ROW + sub * ITEMS;
#pragma unroll
            for (int e = 0; e < ITEMS; ++e)
                if (sub * ITEMS + static_cast<uint32_t>(e) < tail) gp[e] = v[e];
        }
    };
    auto wait1 = [&](uint64_t* bar, uint32_t ph, uint64_t b) -> bool {
        return ptx::mbar_try_wait(bar, ph) || ptx::mbar_wait_bounded(bar, ph, ptx::global_timer_ns() + b);
    };
    // Head-bit words of tile k of queue entry q (segmented scans only).
    auto heads_of = [&](int q, int k) -> uint32_t* { return ctrl->heads[SEG ? q : 0][k]; };
    // Head bits of a thread's ITEMS consecutive items (logical order).
    auto head_bits = [&](const uint32_t* hw, uint32_t thr) -> uint32_t {
        if constexpr (!SEG) {
            return 0u;
        } else if constexpr (ITEMS == 32) {
            return hw[thr];
        } else {
            return (hw[thr * ITEMS / 32] >> ((thr * ITEMS) & 31u)) & ((1u << ITEMS) - 1u);
        }
    };

    // ======================================================== R-loader
    if (warp == 0) {
        if (lane == 0) {
            const uint64_t pol = ptx::policy_evict_last();
            bool stop = false;
            auto acquire = [&]() -> uint64_t { return stop ? ~0ull : atomicAdd(&a.hdr->tile_counter, 1u); };
            auto resolve = [&](uint64_t raw) -> uint32_t {
                if (stop || raw >= num_units || ld_volatile_u32(&a.hdr->error_flags) != 0) {
                    stop = true;
                    return kTileEnd;
                }
                return static_cast<uint32_t>(raw);
            };
            uint32_t rn = 0;
            bool ok = true;
            for (uint32_t i = 0; ok; ++i) {
                const int q = static_cast<int>(i % Q);
                if (i >= Q && !wait1(&ctrl->ufree[q], ((i - Q) / Q) & 1u, long_budget)) break;
                // The unit id is taken only now, when its loads follow, and
                // the unit's full rows are prefetched into L2 (see
                // scan_l2.cuh; measured on GB300: +3-4% for the integer and
                // plain FP32 scans, +2% for the compensated one).
                const uint32_t u = resolve(acquire());
                ctrl->unit_of[q] = u;
                ptx::mbar_arrive(&ctrl->uknown[q]);
                if (u != kTileEnd) {
#pragma unroll
                    for (int k = 0; k < G; ++k) {
                        if (tma_bytes_of(u * G + k) == 0) continue;
                        const uint64_t r0 = static_cast<uint64_t>(u * G + k) * ROWS;
                        const uint64_t r1 = r0 + ROWS < rows_full ? r0 + ROWS : rows_full;
                        ptx::bulk_prefetch_l2(static_cast<const T*>(a.in) + r0 * ROW, static_cast<uint32_t>((r1 - r0) * 128),
                                              pol);
                    }
                }
                if (u == kTileEnd) {
                    for (uint32_t m = 1; m < LW && ok; ++m) {
                        const uint32_t i2 = i + m;
                        const int q2 = static_cast<int>(i2 % Q);
                        if (i2 >= Q && !wait1(&ctrl->ufree[q2], ((i2 - Q) / Q) & 1u, long_budget)) ok = false;
                        if (ok) {
                            ctrl->unit_of[q2] = kTileEnd;
                            ptx::mbar_arrive(&ctrl->uknown[q2]);
                        }
                    }
                    const int s = static_cast<int>(rn % RS);
                    if (ok && (rn < RS || wait1(&ctrl->rfree[s], ((rn - RS) / RS) & 1u, long_budget))) {
                        ctrl->r_tile[s] = kTileEnd;
                        ptx::mbar_arrive(&ctrl->rfull[s]);
                    }
                    break;
                }
                for (int k = 0; k < G && ok; ++k, ++rn) {
                    const int s = static_cast<int>(rn % RS);
                    if (rn >= RS && !wait1(&ctrl->rfree[s], ((rn - RS) / RS) & 1u, long_budget)) {
                        ok = false;
                        break;
                    }
                    const uint32_t t = u * G + k;
                    ctrl->r_tile[s] = t;
                    const uint32_t bytes = tma_bytes_of(t);
                    ptx::mbar_arrive_expect_tx(&ctrl->rfull[s], bytes);
                    if (bytes)
                        ptx::tma_load_2d(rbuf + static_cast<size_t>(s) * TILE, &tin, 0, static_cast<int32_t>(t * ROWS),
                                         &ctrl->rfull[s], pol);
                }
            }
            if (!ok) raise_error(a.hdr, kErrPipelineTimeout);
        }
    }
    // ======================================================== S-loader
    else if (warp == 1) {
        if (lane == 0) {
            const uint64_t pol = ptx::policy_evict_first();
            uint32_t sn = 0;
            bool ok = true;
            for (uint32_t i = 0; ok; ++i) {
                const int q = static_cast<int>(i % Q);
                const uint32_t ph = (i / Q) & 1u;
                if (!wait1(&ctrl->uknown[q], ph, long_budget)) {
                    ok = false;
                    break;
                }
                const uint32_t u = ctrl->unit_of[q];
                const bool end = u == kTileEnd;
                // One unit ahead of the prefix (see scan_l2.cuh).
                if (!end && i >= 1) {
                    const uint32_t ip = i - 1;
                    bool ready = false;
                    const uint64_t deadline = ptx::global_timer_ns() + long_budget;
                    while (!(ready = ptx::mbar_try_wait(&ctrl->uprefix[ip % Q], (ip / Q) & 1u))) {
                        if (ld_volatile_u32(&ctrl->end_seq) <= ip || ptx::global_timer_ns() > deadline) break;
                    }
                    if (!ready) {
                        ok = false;
                        break;
                    }
                }
                for (int k = 0; k < (end ? 1 : G); ++k, ++sn) {
                    const int s = static_cast<int>(sn % SS);
                    if (sn >= SS && !wait1(&ctrl->sfree[s], ((sn - SS) / SS) & 1u, long_budget)) {
                        ok = false;
                        break;
                    }
                    if (end) {
                        ctrl->s_tile[s] = kTileEnd;
                        ptx::mbar_arrive(&ctrl->sfull[s]);
                        break;
                    }
                    const uint32_t t = u * G + k;
                    ctrl->s_tile[s] = t;
                    const uint32_t bytes = tma_bytes_of(t);
                    ptx::mbar_arrive_expect_tx(&ctrl->sfull[s], bytes);
                    if (bytes)
                        ptx::tma_load_2d(sbuf + static_cast<size_t>(s) * TILE, &tin, 0, static_cast<int32_t>(t * ROWS),
                                         &ctrl->sfull[s], pol);
                }
                if (end) break;
            }
            if (!ok) raise_error(a.hdr, kErrPipelineTimeout);
        }
    }
    // ======================================================== storer
    else if (warp == 2) {
        if (lane == 0) {
            const uint64_t pol = ptx::policy_evict_first();
            for (uint32_t sn = 0;; ++sn) {
                const int s = static_cast<int>(sn % SS);
                if (!wait1(&ctrl->sdone[s], (sn / SS) & 1u, long_budget)) {
                    raise_error(a.hdr, kErrPipelineTimeout);
                    break;
                }
                const uint32_t t = ctrl->s_tile[s];
                if (t == kTileEnd) break;
                // Rows past the tensor are clipped by the TMA unit.
                if (tma_bytes_of(t))
                    ptx::tma_store_2d(&tout, 0, static_cast<int32_t>(t * ROWS), sbuf + static_cast<size_t>(s) * TILE,
                                      pol);
                ptx::bulk_commit();
                if (sn >= 1) {
                    ptx::bulk_wait_read<1>();
                    ptx::mbar_arrive(&ctrl->sfree[(sn - 1) % SS]);
                }
            }
            ptx::bulk_wait_all<0>();
            __threadfence();
            const uint32_t prev = atomicAdd(&a.hdr->exit_counter, 1u);
            if (prev == gridDim.x - 1) {
                __threadfence();
                a.hdr->tile_counter = 0;
                a.hdr->exit_counter = 0;
                uint32_t e = epoch + 1;
                if ((e & kEpochMask) == 0) {
                    ptx::u64x2* desc = static_cast<ptx::u64x2*>(a.desc);
                    for (unsigned long long q = 0; q < a.hdr->capacity_tiles * Op::kDescWords; ++q)
                        ptx::st_relaxed_b128(desc + q, ptx::u64x2{0, 0});
                    e += 1;
                }
                __threadfence();
                a.hdr->epoch = e;
            }
        }
    }
    // ======================================================== head warp
    else if (warp == 3) {
        constexpr int kHeadBatch = 8;  // offset loads in flight per lane
        // Unsegmented scans read no head bits; the warp has nothing to do
        // (it must not fall behind the queue phases, so it leaves).
        if constexpr (!SEG) {
            return;
        } else {
            // For each unit of this CTA, marks the elements where a segment
            // starts: the offsets o with tile_start <= o < tile_end, found by a
            // search in the shared samples, then one coalesced read of the
            // sampled block, then a forward walk over the following offsets.
            for (uint32_t i = 0;; ++i) {
                const int q = static_cast<int>(i % Q);
                const uint32_t ph = (i / Q) & 1u;
                bool ok = true;
                if (lane == 0) ok = wait1(&ctrl->uknown[q], ph, long_budget);
                ok = __shfl_sync(kFullMask, ok, 0);
                __syncwarp();
                if (!ok) {
                    if (lane == 0) raise_error(a.hdr, kErrPipelineTimeout);
                    break;
                }
                const uint32_t u = ctrl->unit_of[q];
                if (u == kTileEnd) break;
                for (int k = 0; k < G; ++k)
                    for (int w = lane; w < kHeadWords; w += 32) heads_of(q, k)[w] = 0u;
                __syncwarp();
                if (SEG && nseg != 0) {
                    const uint64_t ustart = static_cast<uint64_t>(u) * G * TILE;
                    const uint64_t uend = min(ustart + static_cast<uint64_t>(G) * TILE, a.n);
                    // First sample greater than ustart (binary search in smem).
                    uint32_t lo_s = 0, hi_s = nsample;  // invariant: sample[lo_s-1] <= ustart < sample[hi_s]
                    while (lo_s < hi_s) {
                        const uint32_t mid = (lo_s + hi_s) >> 1;
                        if (ctrl->sample[mid] <= ustart)
                            lo_s = mid + 1;
                        else
                            hi_s = mid;
                    }
                    // The first offset >= ustart has an index in [lo_i, hi_i].
                    uint32_t lo_i = lo_s == 0 ? 0u : (lo_s - 1) * stride;
                    uint32_t hi_i = lo_s < nsample ? min(lo_s * stride, nseg) : nseg;
                    // Narrow a wide interval (many short segments) 32-fold per
                    // round: one offset per lane, the last lane below ustart wins.
                    while (hi_i - lo_i > kHeadBatch * 32u) {
                        const uint32_t step = (hi_i - lo_i + 31u) / 32u;
                        const uint32_t idx = min(lo_i + lane * step, nseg - 1u);
                        const uint32_t below = __ballot_sync(kFullMask, sg.offsets[idx] < ustart);
                        if (below == 0u) break;  // offsets[lo_i] >= ustart already
                        const uint32_t last = 31u - static_cast<uint32_t>(__clz(below));
                        hi_i = min(lo_i + (last + 1u) * step, hi_i);
                        lo_i = lo_i + last * step;
                    }
                    // Walk forward from lo_i, kHeadBatch loads of 32 offsets in
                    // flight per round, until an offset at or past uend.
                    for (uint32_t cur = lo_i; cur < nseg; cur += kHeadBatch * 32u) {
                        uint32_t o[kHeadBatch];
    #pragma unroll
                        for (int j = 0; j < kHeadBatch; ++j) {
                            const uint32_t idx = cur + static_cast<uint32_t>(j) * 32u + lane;
                            o[j] = idx < nseg ? sg.offsets[idx] : 0xFFFFFFFFu;
                        }
                        bool past = false;
    #pragma unroll
                        for (int j = 0; j < kHeadBatch; ++j) {
                            if (o[j] >= ustart && o[j] < uend) {
                                const uint32_t pos = static_cast<uint32_t>(o[j] - ustart);
                                atomicOr(&heads_of(q, static_cast<int>(pos / TILE))[(pos % TILE) >> 5], 1u << (pos & 31u));
                            }
                            past = past || o[j] >= uend;
                        }
                        if (__any_sync(kFullMask, past)) break;
                    }
                }
                __syncwarp();
                if (lane == 0) ptx::mbar_arrive(&ctrl->uheads[q]);
            }
    
        }
    }
    // ======================================================== lookback
    else if (warp < kWarpAgg) {
        for (uint32_t i = warp - kWarpLookback;; i += LW) {
            const int q = static_cast<int>(i % Q);
            const uint32_t ph = (i / Q) & 1u;
            bool ok = true;
            if (lane == 0) ok = wait1(&ctrl->uknown[q], ph, long_budget);
            ok = __shfl_sync(kFullMask, ok, 0);
            __syncwarp();
            if (!ok) {
                if (lane == 0) raise_error(a.hdr, kErrPipelineTimeout);
                break;
            }
            const uint32_t u = ctrl->unit_of[q];
            if (u == kTileEnd) break;
            const C pre = u == 0 ? Op::chain_zero() : seg_lookback<Op>(a, u, epoch, lane);
            uint32_t state = 0;
            if (lane == 0) {
                const uint64_t deadline = ptx::global_timer_ns() + long_budget;
                while (!ptx::mbar_try_wait(&ctrl->ureduced[q], ph)) {
                    if (ld_volatile_u32(&ctrl->end_seq) <= i) {
                        state = 1;
                        break;
                    }
                    if (ptx::global_timer_ns() > deadline) {
                        state = 2;
                        break;
                    }
                }
            }
            state = __shfl_sync(kFullMask, state, 0);
            __syncwarp();
            if (state != 0) {
                if (lane == 0 && state == 2) raise_error(a.hdr, kErrPipelineTimeout);
                break;
            }
            const C agg = ctrl->uagg[q];
            const bool flag = ctrl->uflag[q] != 0;
            const C incl = flag ? agg : Op::chain_add(pre, agg);
            if (lane == 0) {
                // The last unit of a group passes the group prefix on.
                if ((u % kDetGroupUnits) == kDetGroupUnits - 1)
                    desc_store<Op>(static_cast<ptx::u64x2*>(a.group_desc), u / kDetGroupUnits, desc_words<Op>(a),
                                   kInclusive, false,
                                   epoch, incl);
                ctrl->upre[q] = pre;
                ptx::mbar_arrive(&ctrl->uprefix[q]);
            }
            __syncwarp();
        }
    }
    // ======================================================== aggregator
    // Once per unit: scans the unit's thread aggregates (kLaneEntries per
    // lane, a serial chain, then one warp scan of the lane totals),
    // publishes the unit's aggregate (descriptor, and ureduced for the
    // lookback warp), then leaves each thread's state before
    // it within the unit in place of its aggregate (ustates).
    else if (warp == kWarpAgg) {
        ptx::u64x2* desc = static_cast<ptx::u64x2*>(a.desc);
        for (uint32_t i = 0;; ++i) {
            const int q = static_cast<int>(i % Q);
            const uint32_t ph = (i / Q) & 1u;
            uint32_t state = 0;
            if (lane == 0) {
                const uint64_t deadline = ptx::global_timer_ns() + long_budget;
                while (!ptx::mbar_try_wait(&ctrl->uentries[q], ph)) {
                    if (ld_volatile_u32(&ctrl->end_seq) <= i) {
                        state = 1;
                        break;
                    }
                    if (ptx::global_timer_ns() > deadline) {
                        state = 2;
                        break;
                    }
                }
            }
            state = __shfl_sync(kFullMask, state, 0);
            __syncwarp();
            if (state != 0) {
                if (lane == 0 && state == 2) raise_error(a.hdr, kErrPipelineTimeout);
                break;
            }
            const uint32_t j0 = lane * kLaneEntries;
            S x = Op::zero();
            bool xf = false;
#pragma unroll
            for (uint32_t m = 0; m < kLaneEntries; ++m) {
                const S v = ctrl->tpre[q][entry_at(j0 + m)];
                const bool vf = SEG && ctrl->tflag[SEG ? q : 0][SEG ? j0 + m : 0] != 0;
                seg_combine<Op>(x, xf, v, vf);
            }
            x = Op::norm(x);
            S inc = x;
            bool incf = xf;
            warp_scan_incl<Op, SEG>(inc, incf, lane);
            // The unit's aggregate goes out before the per-thread states.
            const S unit_agg = Op::shfl(inc, 31);
            const bool unit_flag = SEG && __shfl_sync(kFullMask, incf, 31);
            if (lane == 0) {
                const uint32_t u = ctrl->unit_of[q];
                const C chain = Op::to_chain(Op::norm(unit_agg));
                desc_store<Op>(desc, u, desc_words<Op>(a), kAggregate, unit_flag, epoch, chain);
                ctrl->uagg[q] = chain;
                ctrl->uflag[q] = unit_flag;
                ptx::mbar_arrive(&ctrl->ureduced[q]);
            }
            S lp = Op::shfl_up(inc, 1);
            bool lpf = SEG ? __shfl_up_sync(kFullMask, incf, 1) : false;
            if (lane == 0) {
                lp = Op::zero();
                lpf = false;
            }
            // Second pass over the lane's entries: each becomes the state
            // before it, and the chain moves past it.
#pragma unroll
            for (uint32_t m = 0; m < kLaneEntries; ++m) {
                const S v = ctrl->tpre[q][entry_at(j0 + m)];
                const bool vf = SEG && ctrl->tflag[SEG ? q : 0][SEG ? j0 + m : 0] != 0;
                ctrl->tpre[q][entry_at(j0 + m)] = lp;
                if (SEG) ctrl->tflag[SEG ? q : 0][SEG ? j0 + m : 0] = lpf ? 1 : 0;
                seg_combine<Op>(lp, lpf, v, vf);
            }
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&ctrl->ustates[q]);
        }
    }
    // ======================================================== reduce
    // Each thread reduces its part of each tile and leaves the aggregate
    // (and whether its items hold a segment head) for the aggregator; no
    // warp scan and no barrier per tile.
    else if (warp < kWarpFinal) {
        const uint32_t r = tid - kWarpReduce * 32;
        const uint32_t rw = warp - kWarpReduce;
        for (uint32_t rn = 0;; ++rn) {
            const int s = static_cast<int>(rn % RS);
            const uint32_t i = rn / G;
            const int k = static_cast<int>(rn % G);
            const int q = static_cast<int>(i % Q);
            bool ok = ptx::mbar_try_wait(&ctrl->rfull[s], (rn / RS) & 1u) ||
                      ptx::mbar_wait_bounded(&ctrl->rfull[s], (rn / RS) & 1u, ptx::global_timer_ns() + long_budget);
            const uint32_t t = ok ? ctrl->r_tile[s] : kTileEnd;
            const bool live = t != kTileEnd;
            if (SEG && live && k == 0)
                ok = ptx::mbar_try_wait(&ctrl->uheads[q], (i / Q) & 1u) ||
                     ptx::mbar_wait_bounded(&ctrl->uheads[q], (i / Q) & 1u, ptx::global_timer_ns() + long_budget);
            if (!live || !__all_sync(kFullMask, ok)) {
                if (lane == 0) {
                    if (!ok) raise_error(a.hdr, kErrPipelineTimeout);
                    if (rw == 0) *reinterpret_cast<volatile uint32_t*>(&ctrl->end_seq) = i;
                }
                break;
            }
            T v[ITEMS];
            load_row(rbuf + static_cast<size_t>(s) * TILE, t, r, v);
            const uint32_t hb = SEG ? head_bits(heads_of(q, k), r) : 0u;
            const S agg = (SEG && __any_sync(kFullMask, hb != 0u)) ? thread_aggregate<Op, ITEMS, true>(v, hb)
                                                                   : thread_aggregate<Op, ITEMS, false>(v, 0u);
            // Every value of the warp's rows is in registers now.
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&ctrl->rfree[s]);
            const uint32_t j = static_cast<uint32_t>(k) * NROLE + r;
            ctrl->tpre[q][entry_at(j)] = agg;
            if (SEG) ctrl->tflag[SEG ? q : 0][SEG ? j : 0] = hb != 0u ? 1 : 0;
            if (k == G - 1) {
                __syncwarp();
                if (lane == 0) ptx::mbar_arrive(&ctrl->uentries[q]);
            }
        }
    }
    // ======================================================== finalize
    else {
        const uint32_t f = tid - kWarpFinal * 32;
        S run = Op::zero();  // the unit's prefix from the lookback
        for (uint32_t sn = 0;; ++sn) {
            const int s = static_cast<int>(sn % SS);
            const uint32_t i = sn / G;
            const int k = static_cast<int>(sn % G);
            const int q = static_cast<int>(i % Q);
            const bool ok = __all_sync(kFullMask, ptx::mbar_try_wait(&ctrl->sfull[s], (sn / SS) & 1u) ||
                                                      ptx::mbar_wait_bounded(&ctrl->sfull[s], (sn / SS) & 1u,
                                                                             ptx::global_timer_ns() + long_budget));
            const uint32_t t = ok ? ctrl->s_tile[s] : kTileEnd;
            if (t == kTileEnd) {
                if (!ok && lane == 0) raise_error(a.hdr, kErrPipelineTimeout);
                if (lane == 0) ptx::mbar_arrive(&ctrl->sdone[s]);  // lets the storer see the end
                break;
            }
            T* sb = sbuf + static_cast<size_t>(s) * TILE;
            // Scans whose state is wider than an element (the compensated
            // one) keep a single, rolled copy of the per-item chain, the
            // head-aware one: the kernel is sensitive to its code size (every
            // SM sub-partition runs a reduce and a finalize warp next to the
            // other roles). Measured on GB300, 3367 segments of 340 M
            // elements: two unrolled copies (head-free and head-aware) 2.81
            // TB/s, one unrolled head-aware copy 3.43, one copy rolled over
            // chunk pairs 4.69; unsegmented, the rolled chain 6.17 against
            // 5.82 unrolled.
            constexpr bool kRolled = sizeof(S) > sizeof(T);
            T v[ITEMS];
            if constexpr (!kRolled) load_row(sb, t, f, v);
            if (k == 0) {
                // The unit's prefix (which also orders this warp after the
                // head warp's bits), and the per-thread states (ustates).
                bool pok = ptx::mbar_try_wait(&ctrl->uprefix[q], (i / Q) & 1u) ||
                           ptx::mbar_wait_bounded(&ctrl->uprefix[q], (i / Q) & 1u, ptx::global_timer_ns() + long_budget);
                pok = pok && (ptx::mbar_try_wait(&ctrl->ustates[q], (i / Q) & 1u) ||
                              ptx::mbar_wait_bounded(&ctrl->ustates[q], (i / Q) & 1u,
                                                     ptx::global_timer_ns() + long_budget));
                pok = __all_sync(kFullMask, pok);
                if (!pok && lane == 0) raise_error(a.hdr, kErrPipelineTimeout);
                run = Op::from_chain(ctrl->upre[q]);
            }
            const uint32_t hb = SEG ? head_bits(heads_of(q, k), f) : 0u;
            const uint32_t j = static_cast<uint32_t>(k) * NROLE + f;
            const S pre = ctrl->tpre[q][entry_at(j)];
            const bool pf = SEG && ctrl->tflag[SEG ? q : 0][SEG ? j : 0] != 0;
            const S base = pf ? pre : Op::combine(run, pre);
            if constexpr (kRolled) {
                // One head-aware chain, run as a rolled loop over pairs of
                // 16-byte chunks, in place in the stage (or in global memory
                // for the last, partial row).
                const uint32_t rit = f / SPLIT, sub = f % SPLIT;
                const uint64_t row = static_cast<uint64_t>(t) * ROWS + rit;
                S st = base;
                if (row < rows_full) {
                    T* rp = sb + rit * ROW;
#pragma unroll 1
                    for (int cp = 0; cp < CHUNKS; cp += 2) {
                        const int p0 = (static_cast<int>(sub) * CHUNKS + cp) ^ static_cast<int>(rit & 7u);
                        const int p1 = (static_cast<int>(sub) * CHUNKS + cp + 1) ^ static_cast<int>(rit & 7u);
                        Chunk<T> q0 = *reinterpret_cast<const Chunk<T>*>(rp + p0 * EPC);
                        Chunk<T> q1 = *reinterpret_cast<const Chunk<T>*>(rp + p1 * EPC);
                        const uint32_t hbits = hb >> (cp * EPC);
#pragma unroll
                        for (int e = 0; e < 2 * EPC; ++e) {
                            T& x = e < EPC ? q0.v[e] : q1.v[e - EPC];
                            const S before = ((hbits >> e) & 1u) ? Op::zero() : st;
                            st = Op::acc(before, x);
                            x = INCL ? Op::out(st) : Op::out(before);
                        }
                        *reinterpret_cast<Chunk<T>*>(rp + p0 * EPC) = q0;
                        *reinterpret_cast<Chunk<T>*>(rp + p1 * EPC) = q1;
                    }
                } else if (row == rows_full) {
                    const T* gi = static_cast<const T*>(a.in) + row * ROW + sub * ITEMS;
                    T* go = static_cast<T*>(a.out) + row * ROW + sub * ITEMS;
#pragma unroll 1
                    for (uint32_t e = 0; sub * ITEMS + e < tail && e < static_cast<uint32_t>(ITEMS); ++e) {
                        const T x = gi[e];
                        const S before = ((hb >> e) & 1u) ? Op::zero() : st;
                        st = Op::acc(before, x);
                        go[e] = INCL ? Op::out(st) : Op::out(before);
                    }
                }
            } else {
                if (SEG && __any_sync(kFullMask, hb != 0u))
                    thread_outputs<Op, ITEMS, true, INCL>(v, base, hb);
                else
                    thread_outputs<Op, ITEMS, false, INCL>(v, base, 0u);
                store_row(sb, t, f, v);
            }
            ptx::fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) {
                ptx::mbar_arrive(&ctrl->sdone[s]);
                if (k == G - 1) ptx::mbar_arrive(&ctrl->ufree[q]);
            }
        }
    }
}

}  // namespace gps
