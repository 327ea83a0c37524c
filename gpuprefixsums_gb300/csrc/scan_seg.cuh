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
// (dtype per launch: u32, u64, plain FP32, compensated FP32).
//
// Warps: 0 R-loader, 1 S-loader, 2 storer, 3 head warp (segment heads of each
// unit, from the offsets), then LW lookback warps, RW reduce warps and RW
// finalize warps; see scan_l2.cuh for the two passes.
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

// Rotates 16-byte chunks within a thread's items: v'[c] = v[(c - amount) & 7].
template <typename T, int CHUNKS, int EPC>
__device__ __forceinline__ void rotate_chunks(T (&v)[CHUNKS * EPC], uint32_t amount) {
#pragma unroll
    for (int b = 1; b < CHUNKS; b <<= 1) {
        if (amount & b) {
            T t[CHUNKS * EPC];
#pragma unroll
            for (int x = 0; x < CHUNKS * EPC; ++x) t[x] = v[x];
#pragma unroll
            for (int c = 0; c < CHUNKS; ++c)
#pragma unroll
                for (int e = 0; e < EPC; ++e) v[c * EPC + e] = t[((c - b) & (CHUNKS - 1)) * EPC + e];
        }
    }
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

// Per-thread work on a thread's CHUNKS x EPC items. Register chunk c holds
// logical chunk (c + rrot) & (CHUNKS - 1) (the bank-conflict-free read order;
// rrot = 0 when the items were read in logical order). hb holds the items'
// head bits in logical order. Each chunk is summed by its own chain of EPC
// items, so a thread runs CHUNKS short independent chains instead of one long
// one; only the CHUNKS chunk aggregates are then put in logical order.
template <class Op, int CHUNKS, int EPC, bool SEG>
__device__ __forceinline__ uint32_t chunk_head_bits(uint32_t hb, uint32_t c, uint32_t rrot) {
    if (!SEG) return 0u;
    const uint32_t l = (c + rrot) & (CHUNKS - 1);
    return (hb >> (l * EPC)) & ((1u << EPC) - 1u);
}

// Chunk aggregates in logical order; returns the mask (logical order) of the
// chunks that hold a segment head.
template <class Op, int CHUNKS, int EPC, bool SEG, bool REORDER>
__device__ __forceinline__ uint32_t chunk_aggregates(const typename Op::T (&v)[CHUNKS * EPC], uint32_t hb,
                                                     uint32_t rrot, typename Op::S (&ca)[CHUNKS]) {
    using S = typename Op::S;
    uint32_t mask = 0;
#pragma unroll
    for (int c = 0; c < CHUNKS; ++c) {
        const uint32_t bits = chunk_head_bits<Op, CHUNKS, EPC, SEG>(hb, c, rrot);
        S x = Op::zero();
#pragma unroll
        for (int e = 0; e < EPC; ++e) x = ((bits >> e) & 1u) ? Op::lift(v[c * EPC + e]) : Op::acc(x, v[c * EPC + e]);
        ca[c] = x;
        mask |= (bits != 0u ? 1u : 0u) << c;
    }
    if (REORDER) {
        rotate_chunks<S, CHUNKS, 1>(ca, rrot);
        mask = ((mask << rrot) | (mask >> ((CHUNKS - rrot) & (CHUNKS - 1)))) & ((1u << CHUNKS) - 1u);
    }
    return mask;
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

// Sum of a warp's states in every lane, in no particular order (wrapping
// integer sums only).
template <class Op>
__device__ __forceinline__ typename Op::S warp_sum_unordered(typename Op::S s) {
#pragma unroll
    for (int m = 16; m; m >>= 1) s = Op::combine(s, Op::shfl(s, (threadIdx.x & 31u) ^ static_cast<uint32_t>(m)));
    return s;
}

// Thread aggregate of a thread's items and the warp's inclusive scan of it;
// HEADS = false when no item of the warp is a segment head. UNORDERED: only
// the warp total is wanted and the type's sums need no order.
template <class Op, int CHUNKS, int EPC, bool HEADS, bool REORDER, bool UNORDERED>
__device__ __forceinline__ uint32_t thread_and_warp_scan(const typename Op::T (&v)[CHUNKS * EPC], uint32_t hb,
                                                         uint32_t rrot, uint32_t lane, typename Op::S (&ca)[CHUNKS],
                                                         typename Op::S& ws, bool& wf) {
    using S = typename Op::S;
    const uint32_t cmask = chunk_aggregates<Op, CHUNKS, EPC, HEADS, REORDER>(v, hb, rrot, ca);
    S tv = Op::zero();
    bool tf = false;
#pragma unroll
    for (int c = 0; c < CHUNKS; ++c) {
        if (HEADS)
            seg_combine<Op>(tv, tf, ca[c], (cmask >> c) & 1u);
        else
            tv = Op::combine(tv, ca[c]);
    }
    tv = Op::norm(tv);
    if (UNORDERED && !HEADS) {
        tv = warp_sum_unordered<Op>(tv);
    } else {
        warp_scan_incl<Op, HEADS>(tv, tf, lane);
    }
    ws = tv;
    wf = tf;
    return cmask;
}

// Outputs of a thread's items from the state before each chunk (cp, in
// register order): CHUNKS independent chains of EPC items.
template <class Op, int CHUNKS, int EPC, bool SEG, bool INCL>
__device__ __forceinline__ void chunk_outputs(typename Op::T (&v)[CHUNKS * EPC], const typename Op::S (&cp)[CHUNKS],
                                              uint32_t hb, uint32_t rrot) {
    using S = typename Op::S;
#pragma unroll
    for (int c = 0; c < CHUNKS; ++c) {
        const uint32_t bits = chunk_head_bits<Op, CHUNKS, EPC, SEG>(hb, c, rrot);
        S st = cp[c];
#pragma unroll
        for (int e = 0; e < EPC; ++e) {
            const S before = ((bits >> e) & 1u) ? Op::zero() : st;
            st = Op::acc(before, v[c * EPC + e]);
            v[c * EPC + e] = INCL ? Op::out(st) : Op::out(before);
        }
    }
}

// Lookback over 128-bit generic descriptors (see lookback() in
// scan_pipeline.cuh for the scheme): terminators are inclusive prefixes and
// units holding a segment head. Returns the chain value before unit u.
template <class Op>
__device__ typename Op::C seg_lookback(const ScanArgs& a, uint32_t u, uint32_t epoch, uint32_t lane, int64_t bound,
                                       typename Op::C bound_val) {
    using C = typename Op::C;
    constexpr int K = 8;  // 16-byte descriptors per lane per window
    constexpr int WIN = 32 * K;
    constexpr uint32_t kNone = 0xFFFFFFFFu;
    ptx::u64x2* desc = static_cast<ptx::u64x2*>(a.desc);
    C prefix = Op::chain_zero();
    int64_t top = static_cast<int64_t>(u) - 1;
    uint32_t polls = 0;
    uint64_t deadline = 0;
    uint32_t backoff = 64;
    while (true) {
        const int64_t lo = top - WIN + 1;
        auto slot_idx = [&](int j) -> int64_t { return lo + static_cast<int64_t>(j) * 32 + lane; };
        C val[K];
        uint32_t valid = 0, term = 0, pending = 0;
#pragma unroll
        for (int j = 0; j < K; ++j) {
            const int64_t idx = slot_idx(j);
            val[j] = Op::chain_zero();
            if (idx <= bound) {
                valid |= 1u << j;
                term |= 1u << j;
                if (idx == bound) val[j] = bound_val;
            } else {
                pending |= 1u << j;
            }
        }
        while (true) {
#pragma unroll
            for (int j = 0; j < K; ++j) {
                if ((pending >> j) & 1u) {
                    const ptx::u64x2 w = ptx::ld_relaxed_b128(desc + slot_idx(j));
                    const bool ok = (static_cast<uint32_t>(w.hi) & kEpochMask) == (epoch & kEpochMask);
                    const uint32_t st = ok ? static_cast<uint32_t>(w.hi >> 62) : kNotReady;
                    if (st != kNotReady) {
                        valid |= 1u << j;
                        pending &= ~(1u << j);
                        val[j] = Op::chain_from_bits(w.lo);
                        if (st == kInclusive || (w.hi & kHeadFlagBit)) term |= 1u << j;
                    }
                }
            }
            uint32_t my_term = kNone;
#pragma unroll
            for (int j = 0; j < K; ++j)
                if ((term >> j) & 1u) my_term = min(my_term, static_cast<uint32_t>(top - slot_idx(j)));
            const uint32_t pterm = __reduce_min_sync(kFullMask, my_term);
            uint32_t my_gap = kNone;
#pragma unroll
            for (int j = 0; j < K; ++j) {
                const uint32_t pos = static_cast<uint32_t>(top - slot_idx(j));
                if (!((valid >> j) & 1u) && pos < pterm) my_gap = min(my_gap, pos);
            }
            const uint32_t gap = __reduce_min_sync(kFullMask, my_gap);
            if (gap == kNone) {
                C part = Op::chain_zero();
#pragma unroll
                for (int j = 0; j < K; ++j)
                    if (static_cast<uint32_t>(top - slot_idx(j)) <= pterm) part = Op::chain_add(part, val[j]);
                prefix = Op::chain_add(prefix, chain_warp_sum<Op>(part));
                if (pterm != kNone) return prefix;
                top -= WIN;
                polls = 0;
                break;
            }
            ++polls;
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
            __nanosleep(backoff);
            backoff = backoff < 1024 ? backoff * 2 : 1024;
        }
    }
}

template <class Op, int RW, int RS, int SS, int Q, int G, bool SEG>
struct SegCtrl {
    using S = typename Op::S;
    using C = typename Op::C;
    static constexpr int kHeadWords = TileShape<typename Op::T, RW>::kTile / 32;
    uint64_t rfull[RS], rfree[RS];
    uint64_t sfull[SS], sdone[SS], sfree[SS];
    uint64_t uknown[Q], uheads[Q], ureduced[Q], uprefix[Q], ufree[Q];
    uint32_t r_tile[RS];
    uint32_t s_tile[SS];
    uint32_t unit_of[Q];
    uint32_t end_seq;
    uint32_t uflag[Q];  // unit holds a segment head
    C uagg[Q];
    C upre[Q];
    S r_wtot[2][RW];
    uint32_t r_wflag[2][RW];
    S f_wtot[2][RW];
    uint32_t f_wflag[2][RW];
    // Segmented scans only (one unused entry otherwise):
    uint32_t heads[SEG ? Q : 1][G][kHeadWords];  // bit b of word w: element 32w+b is a segment head
    uint32_t sample[SEG ? 1024 : 1];             // offsets[j * sample_stride], to start head searches
};

template <class Op, int RW, int RS, int SS, int Q, int G, bool SEG>
constexpr size_t seg_smem_bytes() {
    return static_cast<size_t>(RS + SS) * TileShape<typename Op::T, RW>::kTile * sizeof(typename Op::T) +
           sizeof(SegCtrl<Op, RW, RS, SS, Q, G, SEG>);
}

template <class Op, int RW>
struct SegShape {
    static constexpr int kLookbackWarps = 3;
    static constexpr int kThreads = 32 * (4 + kLookbackWarps + 2 * RW);
};

template <class Op, int RW, int RS, int SS, int Q, int G, bool INCL, bool SEG>
__global__ void __launch_bounds__(SegShape<Op, RW>::kThreads, 1) scan_seg_kernel(const ScanArgs a, const SegArgs sg) {
    using T = typename Op::T;
    using S = typename Op::S;
    using C = typename Op::C;
    using Shape = TileShape<T, RW>;
    constexpr int TILE = Shape::kTile;
    constexpr int ITEMS = Shape::kItems;
    constexpr int EPC = 16 / static_cast<int>(sizeof(T));
    constexpr int CHUNKS = ITEMS / EPC;
    constexpr uint32_t NROLE = Shape::kRoleThreads;
    constexpr uint32_t LW = SegShape<Op, RW>::kLookbackWarps;
    constexpr uint32_t kWarpLookback = 4, kWarpReduce = 4 + LW, kWarpFinal = 4 + LW + RW;
    constexpr int kHeadWords = TILE / 32;
    static_assert(CHUNKS == 8, "128 bytes per thread");
    static_assert(Q > LW, "every lookback warp needs its own queue entry");
    using Ctrl = SegCtrl<Op, RW, RS, SS, Q, G, SEG>;
    // The reduce pass sums the chunk aggregates in logical order for
    // segmented scans (heads) and for floating point (the summation order of
    // the scan pass); wrapping integer sums need no order.
    constexpr bool REORDER = SEG || !std::is_integral<T>::value;

    extern __shared__ __align__(1024) uint8_t smem_raw[];
    T* rbuf = reinterpret_cast<T*>(smem_raw);
    T* sbuf = rbuf + static_cast<size_t>(RS) * TILE;
    Ctrl* ctrl = reinterpret_cast<Ctrl*>(smem_raw + static_cast<size_t>(RS + SS) * TILE * sizeof(T));

    const uint32_t tid = threadIdx.x;
    const uint32_t warp = tid >> 5;
    const uint32_t lane = tid & 31u;
    const uint32_t num_units = (a.num_tiles + G - 1) / G;
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
            ptx::mbar_init(&ctrl->ureduced[q], 1);
            ptx::mbar_init(&ctrl->uprefix[q], 1);
            ptx::mbar_init(&ctrl->ufree[q], RW);
        }
        ctrl->end_seq = 0xFFFFFFFFu;
        ptx::fence_mbar_init();
    }
    if (SEG)
        for (uint32_t j = tid; j < nsample; j += blockDim.x) ctrl->sample[j] = sg.offsets[min(j * stride, nseg)];
    __syncthreads();

    const uint32_t epoch = ld_volatile_u32(&a.hdr->epoch);
    const uint64_t budget = a.wait_budget_ns;
    const uint64_t long_budget = budget * 4 + 1000000000ull;
    auto count_of = [&](uint32_t t) -> uint32_t { return t < a.num_tiles ? tile_count<TILE>(a.n, t) : 0u; };
    auto bulk_bytes_of = [&](uint32_t t) -> uint32_t {
        return (count_of(t) * static_cast<uint32_t>(sizeof(T))) & ~15u;
    };
    auto wait1 = [&](uint64_t* bar, uint32_t ph, uint64_t b) -> bool {
        return ptx::mbar_try_wait(bar, ph) || ptx::mbar_wait_bounded(bar, ph, ptx::global_timer_ns() + b);
    };
    // Head-bit words of tile k of queue entry q (segmented scans only).
    auto heads_of = [&](int q, int k) -> uint32_t* { return ctrl->heads[SEG ? q : 0][k]; };
    // Head bits of a thread's ITEMS consecutive items (logical order).
    auto head_bits = [&](const uint32_t* hw, uint32_t thr) -> uint32_t {
        if (!SEG) return 0u;
        if (ITEMS == 32) return hw[thr];
        return (hw[thr * ITEMS / 32] >> ((thr * ITEMS) & 31u)) & ((1u << ITEMS) - 1u);
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
                // The unit id is taken only now, when its loads follow (see
                // scan_l2.cuh). No L2 prefetch here: this kernel is bound by
                // its per-tile work, and the prefetched lines only crowd the
                // L2 (measured: 7% slower on the 4096-segment batch).
                const uint32_t u = resolve(acquire());
                ctrl->unit_of[q] = u;
                ptx::mbar_arrive(&ctrl->uknown[q]);
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
                    const uint32_t bytes = bulk_bytes_of(t);
                    ptx::mbar_arrive_expect_tx(&ctrl->rfull[s], bytes);
                    if (bytes)
                        ptx::bulk_load_hint(rbuf + static_cast<size_t>(s) * TILE,
                                            static_cast<const T*>(a.in) + static_cast<uint64_t>(t) * TILE, bytes,
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
                    const uint32_t bytes = bulk_bytes_of(t);
                    ptx::mbar_arrive_expect_tx(&ctrl->sfull[s], bytes);
                    if (bytes)
                        ptx::bulk_load_hint(sbuf + static_cast<size_t>(s) * TILE,
                                            static_cast<const T*>(a.in) + static_cast<uint64_t>(t) * TILE, bytes,
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
                const uint32_t bytes = bulk_bytes_of(t);
                if (bytes)
                    ptx::bulk_store_hint(static_cast<T*>(a.out) + static_cast<uint64_t>(t) * TILE,
                                         sbuf + static_cast<size_t>(s) * TILE, bytes, pol);
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
                    for (unsigned long long q = 0; q < a.hdr->capacity_tiles; ++q)
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
        if (!SEG) return;
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
    // ======================================================== lookback
    else if (warp < kWarpReduce) {
        ptx::u64x2* desc = static_cast<ptx::u64x2*>(a.desc);
        int64_t own_prev = -1;
        C own_incl = Op::chain_zero();
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
            const C pre = u == 0 ? Op::chain_zero() : seg_lookback<Op>(a, u, epoch, lane, own_prev, own_incl);
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
                if (u != 0) ptx::st_relaxed_b128(desc + u, seg_pack(kInclusive, flag, epoch, Op::chain_bits(incl)));
                ctrl->upre[q] = pre;
                ptx::mbar_arrive(&ctrl->uprefix[q]);
            }
            own_prev = u;
            own_incl = incl;
            __syncwarp();
        }
    }
    // ======================================================== reduce
    else if (warp < kWarpFinal) {
        const uint32_t r = tid - kWarpReduce * 32;
        const uint32_t rw = warp - kWarpReduce;
        const uint32_t rot = r & 7u;
        ptx::u64x2* desc = static_cast<ptx::u64x2*>(a.desc);
        S unit_agg = Op::zero();
        bool unit_flag = false;
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
            const T* sb = rbuf + static_cast<size_t>(s) * TILE;
            const uint32_t cnt = live ? count_of(t) : 0u;
            T v[ITEMS];
            if (cnt == static_cast<uint32_t>(TILE)) {
#pragma unroll
                for (int c8 = 0; c8 < CHUNKS; ++c8) {
                    const uint32_t c = (c8 + rot) & (CHUNKS - 1);
                    const Chunk<T> qv = *reinterpret_cast<const Chunk<T>*>(sb + r * ITEMS + c * EPC);
#pragma unroll
                    for (int e = 0; e < EPC; ++e) v[c8 * EPC + e] = qv.v[e];
                }
            } else {
                const uint32_t bulk_elems = live ? bulk_bytes_of(t) / static_cast<uint32_t>(sizeof(T)) : 0u;
                const uint64_t gbase = static_cast<uint64_t>(live ? t : 0u) * TILE;
#pragma unroll
                for (int e = 0; e < ITEMS; ++e) {
                    const uint32_t li = r * ITEMS + e;
                    T x = T(0);
                    if (li < bulk_elems)
                        x = sb[li];
                    else if (li < cnt)
                        x = static_cast<const T*>(a.in)[gbase + li];
                    v[e] = x;
                }
            }
            const uint32_t hb = (SEG && live) ? head_bits(heads_of(q, k), r) : 0u;
            const uint32_t rrot = cnt == static_cast<uint32_t>(TILE) ? rot : 0u;
            // Warp aggregate (items beyond cnt are zero and carry no head),
            // formed exactly as the finalize warps form it for floating point:
            // chunk aggregates in logical order, then a lane-order scan. Warps
            // whose items hold no segment head take the plain path.
            S ca[CHUNKS];
            S tv;
            bool tf;
            if (SEG && __any_sync(kFullMask, hb != 0u))
                thread_and_warp_scan<Op, CHUNKS, EPC, SEG, REORDER, false>(v, hb, rrot, lane, ca, tv, tf);
            else
                thread_and_warp_scan<Op, CHUNKS, EPC, false, !std::is_integral<T>::value,
                                     std::is_integral<T>::value>(v, 0u, rrot, lane, ca, tv, tf);
            if (lane == 31) {
                ctrl->r_wtot[rn & 1u][rw] = tv;
                ctrl->r_wflag[rn & 1u][rw] = tf;
            }
            const bool stop = named_bar_or(1, NROLE, !live || !ok);
            if (lane == 0 && live) ptx::mbar_arrive(&ctrl->rfree[s]);
            if (stop) {
                if (r == 0) {
                    if (!ok) raise_error(a.hdr, kErrPipelineTimeout);
                    *reinterpret_cast<volatile uint32_t*>(&ctrl->end_seq) = i;
                }
                break;
            }
            if (r == 0) {
                S agg = Op::zero();
                bool af = false;
#pragma unroll
                for (int w2 = 0; w2 < RW; ++w2)
                    seg_combine<Op>(agg, af, ctrl->r_wtot[rn & 1u][w2], ctrl->r_wflag[rn & 1u][w2] != 0);
                seg_combine<Op>(unit_agg, unit_flag, agg, af);
                if (k == G - 1) {
                    const uint32_t u = t / G;
                    const C chain = Op::to_chain(unit_agg);
                    ptx::st_relaxed_b128(desc + u, seg_pack(u == 0 ? kInclusive : kAggregate, unit_flag, epoch,
                                                            Op::chain_bits(chain)));
                    ctrl->uagg[q] = chain;
                    ctrl->uflag[q] = unit_flag;
                    ptx::mbar_arrive(&ctrl->ureduced[q]);
                    unit_agg = Op::zero();
                    unit_flag = false;
                }
            }
        }
    }
    // ======================================================== finalize
    else {
        const uint32_t f = tid - kWarpFinal * 32;
        const uint32_t fw = warp - kWarpFinal;
        const uint32_t rot = f & 7u;
        S run = Op::zero();  // state before the current tile
        bool go = true;
        for (uint32_t sn = 0; go; ++sn) {
            const int s = static_cast<int>(sn % SS);
            const uint32_t i = sn / G;
            const int k = static_cast<int>(sn % G);
            const int q = static_cast<int>(i % Q);
            const bool ok = ptx::mbar_try_wait(&ctrl->sfull[s], (sn / SS) & 1u) ||
                            ptx::mbar_wait_bounded(&ctrl->sfull[s], (sn / SS) & 1u, ptx::global_timer_ns() + long_budget);
            const uint32_t t = ok ? ctrl->s_tile[s] : kTileEnd;
            const bool live = t != kTileEnd;
            T* sb = sbuf + static_cast<size_t>(s) * TILE;
            const uint32_t cnt = live ? count_of(t) : 0u;
            const bool full_tile = cnt == static_cast<uint32_t>(TILE);
            const uint32_t bulk_elems = live ? bulk_bytes_of(t) / static_cast<uint32_t>(sizeof(T)) : 0u;
            const uint64_t gbase = static_cast<uint64_t>(live ? t : 0u) * TILE;
            T v[ITEMS];
            if (full_tile) {
#pragma unroll
                for (int c8 = 0; c8 < CHUNKS; ++c8) {
                    const uint32_t c = (c8 + rot) & (CHUNKS - 1);
                    const Chunk<T> qv = *reinterpret_cast<const Chunk<T>*>(sb + f * ITEMS + c * EPC);
#pragma unroll
                    for (int e = 0; e < EPC; ++e) v[c8 * EPC + e] = qv.v[e];
                }
            } else {
#pragma unroll
                for (int e = 0; e < ITEMS; ++e) {
                    const uint32_t li = f * ITEMS + e;
                    T x = T(0);
                    if (li < bulk_elems)
                        x = sb[li];
                    else if (li < cnt)
                        x = static_cast<const T*>(a.in)[gbase + li];
                    v[e] = x;
                }
            }
            // The head warp may still be marking this unit: wait for it (its
            // bits stay valid until this unit's queue entry is released).
            bool hok = true;
            if (SEG && live && k == 0)
                hok = ptx::mbar_try_wait(&ctrl->uheads[q], (i / Q) & 1u) ||
                      ptx::mbar_wait_bounded(&ctrl->uheads[q], (i / Q) & 1u, ptx::global_timer_ns() + long_budget);
            if (!hok) raise_error(a.hdr, kErrPipelineTimeout);
            const uint32_t hb = (SEG && live) ? head_bits(heads_of(q, k), f) : 0u;
            const uint32_t rrot = full_tile ? rot : 0u;
            // Chunk aggregates (logical order) and the warp's inclusive scan
            // of the thread aggregates; then exclusive by one lane.
            S ca[CHUNKS];
            S wv;
            bool wf;
            const bool heads_here = SEG && __any_sync(kFullMask, hb != 0u);
            const uint32_t cmask =
                heads_here ? thread_and_warp_scan<Op, CHUNKS, EPC, SEG, true, false>(v, hb, rrot, lane, ca, wv, wf)
                           : thread_and_warp_scan<Op, CHUNKS, EPC, false, true, false>(v, 0u, rrot, lane, ca, wv, wf);
            S xv = Op::shfl_up(wv, 1);
            bool xf = SEG ? __shfl_up_sync(kFullMask, wf, 1) : false;
            if (lane == 0) {
                xv = Op::zero();
                xf = false;
            }
            if (lane == 31) {
                ctrl->f_wtot[sn & 1u][fw] = wv;
                ctrl->f_wflag[sn & 1u][fw] = wf;
            }
            if (named_bar_or(2, NROLE, !live)) {
                if (!ok && f == 0) raise_error(a.hdr, kErrPipelineTimeout);
                if (lane == 0) ptx::mbar_arrive(&ctrl->sdone[s]);
                go = false;
                break;
            }
            if (k == 0) {
                bool pok = ptx::mbar_try_wait(&ctrl->uprefix[q], (i / Q) & 1u) ||
                           ptx::mbar_wait_bounded(&ctrl->uprefix[q], (i / Q) & 1u, ptx::global_timer_ns() + long_budget);
                pok = __all_sync(kFullMask, pok);
                if (!pok && lane == 0) raise_error(a.hdr, kErrPipelineTimeout);
                run = Op::from_chain(ctrl->upre[q]);
            }
            // State before this thread: tile prefix, earlier warps, earlier lanes.
            S base = run;
            bool bf = false;
            S tile_agg = Op::zero();
            bool tile_f = false;
#pragma unroll
            for (int w2 = 0; w2 < RW; ++w2) {
                const S x = ctrl->f_wtot[sn & 1u][w2];
                const bool xfl = ctrl->f_wflag[sn & 1u][w2] != 0;
                if (static_cast<uint32_t>(w2) < fw) seg_combine<Op>(base, bf, x, xfl);
                seg_combine<Op>(tile_agg, tile_f, x, xfl);
            }
            seg_combine<Op>(base, bf, xv, xf);
            {
                bool rf = false;
                seg_combine<Op>(run, rf, tile_agg, tile_f);
            }
            // State before each chunk (logical order), then back to register
            // order; then CHUNKS independent chains of EPC items.
            {
                S st = base;
                bool sf = false;
#pragma unroll
                for (int c = 0; c < CHUNKS; ++c) {
                    const S x = ca[c];
                    ca[c] = st;
                    seg_combine<Op>(st, sf, x, (cmask >> c) & 1u);
                }
            }
            rotate_chunks<S, CHUNKS, 1>(ca, (CHUNKS - rrot) & (CHUNKS - 1));
            if (heads_here)
                chunk_outputs<Op, CHUNKS, EPC, SEG, INCL>(v, ca, hb, rrot);
            else
                chunk_outputs<Op, CHUNKS, EPC, false, INCL>(v, ca, 0u, rrot);
            if (full_tile) {
#pragma unroll
                for (int c8 = 0; c8 < CHUNKS; ++c8) {
                    const uint32_t c = (c8 + rot) & (CHUNKS - 1);
                    Chunk<T> qv;
#pragma unroll
                    for (int e = 0; e < EPC; ++e) qv.v[e] = v[c8 * EPC + e];
                    *reinterpret_cast<Chunk<T>*>(sb + f * ITEMS + c * EPC) = qv;
                }
            } else {
#pragma unroll
                for (int e = 0; e < ITEMS; ++e) {
                    const uint32_t li = f * ITEMS + e;
                    if (li < bulk_elems)
                        sb[li] = v[e];
                    else if (li < cnt)
                        static_cast<T*>(a.out)[gbase + li] = v[e];
                }
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
