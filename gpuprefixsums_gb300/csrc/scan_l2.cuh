// Single-pass chained scan that buffers in L2 (sm_103a), for 16-byte-aligned
// buffers.
//
// Every tile is read twice but fetched from HBM once:
//   reduce pass  prefetch the unit into L2 when its id is taken, then
//                bulk-load each tile into a shared-memory ring with an
//                L2 evict-last policy, sum it, free the stage at once, and
//                publish each unit's aggregate (a unit is G tiles taken by
//                one CTA);
//   scan pass    when the unit's prefix is (about to be) known, bulk-load the
//                tile again -- from L2, evict-first -- scan it, add the
//                prefix and bulk-store it.
// HBM sees one read and one write per element, like the single-pass scan of
// the reference (ChainedScanDecoupledLookback.cuh:79-139), but the time a tile
// waits for its lookback is spent in the 129 MB L2 instead of in shared
// memory, so the shared-memory ring only covers load latency and the lookback
// never throttles the stream.
//
// Warps of a CTA (one CTA per SM):
//   0          R-loader  takes unit ids (atomic counter), issues reduce-pass loads
//   1          S-loader  issues scan-pass loads of a unit once the previous
//                        unit's prefix is known
//   2          storer    bulk-stores scanned tiles, frees scan stages
//   3..2+LW    lookback  resolve unit prefixes (alternate units), starting as
//                        soon as a unit id is known
//   RW warps   reduce    sum reduce-pass tiles, publish unit aggregates
//   RW warps   finalize  scan scan-pass tiles with the unit prefix
// Hand-off is through mbarriers; every wait is bounded by the plan's budget.
#pragma once
#include "scan_pipeline.cuh"

namespace gps {

template <typename T, int RW, int RS, int SS, int Q, int G>
struct L2Ctrl {
    uint64_t rfull[RS];     // R-loader -> reduce: tile landed
    uint64_t rfree[RS];     // reduce -> R-loader: stage read
    uint64_t sfull[SS];     // S-loader -> finalize: tile landed
    uint64_t sdone[SS];     // finalize -> storer: tile scanned in place
    uint64_t sfree[SS];     // storer -> S-loader: store has read the stage
    uint64_t uknown[Q];     // R-loader -> lookback, S-loader: unit id set
    uint64_t ureduced[Q];   // reduce -> lookback, S-loader: unit aggregate set
    uint64_t uprefix[Q];    // lookback -> S-loader, finalize: unit prefix set
    uint64_t ufree[Q];      // finalize -> R-loader: queue entry reusable
    uint32_t r_tile[RS];
    uint32_t s_tile[SS];
    uint32_t unit_of[Q];
    uint32_t end_seq;       // first unit sequence number the reduce warps did not take
    T uagg[Q];
    T upre[Q];
    T r_warp_tot[2][RW];  // inclusive warp totals of the reduce pass
    // Exclusive prefix of each reduce/finalize thread's 128 bytes within its
    // unit, from the reduce pass: the scan pass then needs no cross-warp
    // exchange (no warp scan, no barrier) per tile.
    T tpre[Q][G][RW * 32];
};

template <typename T, int RW, int RS, int SS, int Q, int G>
constexpr size_t l2_smem_bytes() {
    return static_cast<size_t>(RS + SS) * TileShape<T, RW>::kTile * sizeof(T) + sizeof(L2Ctrl<T, RW, RS, SS, Q, G>);
}

template <typename T, int RW>
struct L2Shape {
    static constexpr int kLookbackWarps = 3;
    static constexpr int kThreads = 32 * (3 + kLookbackWarps + 2 * RW);
};

template <typename T, int RW, int RS, int SS, int Q, int G, bool INCL, bool STALL>
__global__ void __launch_bounds__(L2Shape<T, RW>::kThreads, 1) scan_l2_kernel(const ScanArgs a) {
    using Shape = TileShape<T, RW>;
    constexpr int TILE = Shape::kTile;
    constexpr int ITEMS = Shape::kItems;
    constexpr int EPC = 16 / static_cast<int>(sizeof(T));
    constexpr int CHUNKS = ITEMS / EPC;
    constexpr uint32_t NROLE = Shape::kRoleThreads;
    constexpr uint32_t LW = L2Shape<T, RW>::kLookbackWarps;
    constexpr uint32_t kWarpLookback = 3, kWarpReduce = 3 + LW, kWarpFinal = 3 + LW + RW;
    static_assert(CHUNKS == 8, "128 bytes per thread");
    static_assert(Q > LW, "every lookback warp needs its own queue entry");
    using D = DescTraits<T>;
    using word = typename D::word;
    using Ctrl = L2Ctrl<T, RW, RS, SS, Q, G>;

    extern __shared__ __align__(1024) uint8_t smem_raw[];
    T* rbuf = reinterpret_cast<T*>(smem_raw);
    T* sbuf = rbuf + static_cast<size_t>(RS) * TILE;
    Ctrl* ctrl = reinterpret_cast<Ctrl*>(smem_raw + static_cast<size_t>(RS + SS) * TILE * sizeof(T));

    const uint32_t tid = threadIdx.x;
    const uint32_t warp = tid >> 5;
    const uint32_t lane = tid & 31u;
    const uint32_t num_units = (a.num_tiles + G - 1) / G;

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
            ptx::mbar_init(&ctrl->ureduced[q], 1);
            ptx::mbar_init(&ctrl->uprefix[q], 1);
            ptx::mbar_init(&ctrl->ufree[q], RW);
        }
        ctrl->end_seq = 0xFFFFFFFFu;
        ptx::fence_mbar_init();
    }
    __syncthreads();

    const uint32_t epoch = ld_volatile_u32(&a.hdr->epoch);
    const T carry = a.carry_in != nullptr ? *static_cast<const T*>(a.carry_in) : T(0);
    const uint64_t budget = a.wait_budget_ns;
    const uint64_t long_budget = budget * 4 + 1000000000ull;
    auto count_of = [&](uint32_t t) -> uint32_t { return t < a.num_tiles ? tile_count<TILE>(a.n, t) : 0u; };
    auto bulk_bytes_of = [&](uint32_t t) -> uint32_t {
        return (count_of(t) * static_cast<uint32_t>(sizeof(T))) & ~15u;
    };
    // Single-thread bounded wait; false once the budget has run out.
    auto wait1 = [&](uint64_t* bar, uint32_t ph, uint64_t b) -> bool {
        return ptx::mbar_try_wait(bar, ph) || ptx::mbar_wait_bounded(bar, ph, ptx::global_timer_ns() + b);
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
            uint32_t rn = 0;  // reduce-stage uses so far
            bool ok = true;
            for (uint32_t i = 0; ok; ++i) {
                const int q = static_cast<int>(i % Q);
                if (i >= Q && !wait1(&ctrl->ufree[q], ((i - Q) / Q) & 1u, long_budget)) break;
                // The unit id is taken only now, when its queue entry is free
                // and its loads follow: the later an id is taken, the sooner
                // after it the unit's aggregate is published for the units
                // after it (measured: 1.4% faster than taking it one unit
                // ahead).
                const uint32_t u = resolve(acquire());
                ctrl->unit_of[q] = u;
                ptx::mbar_arrive(&ctrl->uknown[q]);
                // Start the unit's HBM reads now, into L2 (evict-last): its
                // shared-memory loads below wait for free stages, and find
                // the data in L2 instead of paying the HBM latency then.
                // This keeps more bytes in flight than the stage ring holds
                // (measured: 5.90 -> 6.20 TB/s at 2^28).
                if (u != kTileEnd) {
#pragma unroll
                    for (int k = 0; k < G; ++k) {
                        const uint32_t bb = bulk_bytes_of(u * G + k);
                        if (bb)
                            ptx::bulk_prefetch_l2(static_cast<const T*>(a.in) + static_cast<uint64_t>(u * G + k) * TILE,
                                                  bb, pol);
                    }
                }
                if (u == kTileEnd) {
                    // The other lookback warps wait on the next entries.
                    for (uint32_t m = 1; m < LW && ok; ++m) {
                        const uint32_t i2 = i + m;
                        const int q2 = static_cast<int>(i2 % Q);
                        if (i2 >= Q && !wait1(&ctrl->ufree[q2], ((i2 - Q) / Q) & 1u, long_budget)) ok = false;
                        if (ok) {
                            ctrl->unit_of[q2] = kTileEnd;
                            ptx::mbar_arrive(&ctrl->uknown[q2]);
                        }
                    }
                    // The reduce warps stop at an empty stage.
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
                // Load the unit again once the previous unit's prefix is
                // known: its own lookback then usually completes while its
                // tiles come back from L2 (they were loaded, and reduced, well
                // before), and the scan-pass stages hold at most one unit
                // that waits for its prefix; any longer wait is spent in L2.
                // Entry i - 1 cannot have been reused yet: the finalize warps
                // still need the tiles of unit i - 1 this thread just issued.
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
                    // Free the previous stage once its store has read it.
                    ptx::bulk_wait_read<1>();
                    ptx::mbar_arrive(&ctrl->sfree[(sn - 1) % SS]);
                }
            }
            ptx::bulk_wait_all<0>();
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
    }
    // ======================================================== lookback
    else if (warp < kWarpReduce) {
        word* desc = static_cast<word*>(a.desc);
        int64_t own_prev = -1;  // last unit this warp resolved, and its inclusive prefix
        T own_incl = 0;
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
            // Walk back while this unit's own tiles are still streaming in.
            const T pre = u == 0 ? carry : lookback<T, TILE * G, STALL>(a, u, epoch, lane, carry, own_prev, own_incl);
            uint32_t state = 0;  // 0 reduced, 1 reduce warps stopped, 2 timeout
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
            const T agg = ctrl->uagg[q];
            if (lane == 0) {
                if (STALL) {
                    // In place, a unit's output may only be written after its
                    // aggregate is in its descriptor: a successor's fallback
                    // re-reads its input (EmulatedDeadlocking.cuh:113-133).
                    const uint64_t deadline = ptx::global_timer_ns() + long_budget;
                    while (D::status(D::load(desc + u), epoch) == kNotReady && ptx::global_timer_ns() < deadline)
                        __nanosleep(200);
                    __threadfence();
                }
                if (u != 0) D::store(desc + u, D::pack(kInclusive, epoch, pre + agg));
                if (a.carry_out != nullptr && u == num_units - 1) *static_cast<T*>(a.carry_out) = pre + agg;
                ctrl->upre[q] = pre;
                ptx::mbar_arrive(&ctrl->uprefix[q]);
            }
            own_prev = u;
            own_incl = pre + agg;
            __syncwarp();
        }
    }
    // ======================================================== reduce
    else if (warp < kWarpFinal) {
        const uint32_t r = tid - kWarpReduce * 32;
        const uint32_t rw = warp - kWarpReduce;
        const uint32_t rot = r & 7u;
        word* desc = static_cast<word*>(a.desc);
        T unit_agg = 0;
        for (uint32_t rn = 0;; ++rn) {
            const int s = static_cast<int>(rn % RS);
            const bool ok = ptx::mbar_try_wait(&ctrl->rfull[s], (rn / RS) & 1u) ||
                            ptx::mbar_wait_bounded(&ctrl->rfull[s], (rn / RS) & 1u, ptx::global_timer_ns() + budget);
            const uint32_t t = ok ? ctrl->r_tile[s] : kTileEnd;
            const bool live = t != kTileEnd;
            const T* sb = rbuf + static_cast<size_t>(s) * TILE;
            const uint32_t cnt = live ? count_of(t) : 0u;
            T total = 0;
            if (cnt == static_cast<uint32_t>(TILE)) {
#pragma unroll
                for (int c8 = 0; c8 < CHUNKS; ++c8) {
                    const uint32_t c = (c8 + rot) & (CHUNKS - 1);
                    const Chunk<T> qv = *reinterpret_cast<const Chunk<T>*>(sb + r * ITEMS + c * EPC);
#pragma unroll
                    for (int e = 0; e < EPC; ++e) total += qv.v[e];
                }
            } else if (cnt != 0) {
                const uint32_t bulk_elems = bulk_bytes_of(t) / static_cast<uint32_t>(sizeof(T));
                const uint64_t gbase = static_cast<uint64_t>(t) * TILE;
#pragma unroll 4
                for (int e = 0; e < ITEMS; ++e) {
                    const uint32_t li = r * ITEMS + e;
                    if (li < bulk_elems)
                        total += sb[li];
                    else if (li < cnt)
                        total += static_cast<const T*>(a.in)[gbase + li];
                }
            }
            const T winc = warp_inclusive_scan(total, lane);
            if (lane == 31) ctrl->r_warp_tot[rn & 1u][rw] = winc;
            const bool stop = named_bar_or(1, NROLE, !live);
            // The stage has been read by every reduce thread.
            if (lane == 0 && live) ptx::mbar_arrive(&ctrl->rfree[s]);
            if (stop) {
                if (r == 0) {
                    if (!ok) raise_error(a.hdr, kErrPipelineTimeout);
                    *reinterpret_cast<volatile uint32_t*>(&ctrl->end_seq) = rn / G;
                }
                break;
            }
            {
                // This thread's prefix within the unit, for the scan pass.
                T wpre = 0, agg = 0;
#pragma unroll
                for (int w2 = 0; w2 < RW; ++w2) {
                    const T x = ctrl->r_warp_tot[rn & 1u][w2];
                    wpre += (static_cast<uint32_t>(w2) < rw) ? x : T(0);
                    agg += x;
                }
                ctrl->tpre[(rn / G) % Q][rn % G][r] = unit_agg + wpre + (winc - total);
                unit_agg += agg;
            }
            if (r == 0) {
                if ((t % G) == G - 1) {
                    const uint32_t u = t / G;
                    const int q = static_cast<int>((rn / G) % Q);
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
                    // Only unit 0's value is an inclusive prefix, so only it
                    // holds the carry. A rescuer computes the same integer
                    // aggregate, so a plain store over an inserted one is
                    // harmless; rescuers use a CAS so that they never
                    // overwrite an inclusive prefix.
                    if (publish)
                        D::store(desc + u, u == 0 ? D::pack(kInclusive, epoch, carry + unit_agg)
                                                  : D::pack(kAggregate, epoch, unit_agg));
                    ctrl->uagg[q] = unit_agg;
                    ptx::mbar_arrive(&ctrl->ureduced[q]);
                }
            }
            if ((rn % G) == G - 1) unit_agg = 0;
        }
    }
    // ======================================================== finalize
    else {
        const uint32_t f = tid - kWarpFinal * 32;
        const uint32_t rot = f & 7u;
        T run = 0;
        bool go = true;
        for (uint32_t sn = 0; go; ++sn) {
            const int s = static_cast<int>(sn % SS);
            const uint32_t i = sn / G;  // unit sequence number
            const int q = static_cast<int>(i % Q);
            const bool ok = __all_sync(kFullMask, ptx::mbar_try_wait(&ctrl->sfull[s], (sn / SS) & 1u) ||
                                                      ptx::mbar_wait_bounded(&ctrl->sfull[s], (sn / SS) & 1u,
                                                                             ptx::global_timer_ns() + long_budget));
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
                    // Logical order for partial tiles.
                    const uint32_t li = f * ITEMS + e;
                    T x = 0;
                    if (li < bulk_elems)
                        x = sb[li];
                    else if (li < cnt)
                        x = static_cast<const T*>(a.in)[gbase + li];
                    v[e] = x;
                }
            }
            if (!live) {
                if (!ok && f == 0) raise_error(a.hdr, kErrPipelineTimeout);
                if (lane == 0) ptx::mbar_arrive(&ctrl->sdone[s]);  // lets the storer see the end
                go = false;
                break;
            }
            T cs[CHUNKS];
#pragma unroll
            for (int c8 = 0; c8 < CHUNKS; ++c8) {
                T x = 0;
#pragma unroll
                for (int e = 0; e < EPC; ++e) x += v[c8 * EPC + e];
                cs[c8] = x;
            }
            T cpre[CHUNKS];
            T total;
            rotated_chunk_prefix<T, CHUNKS>(cs, full_tile ? rot : 0u, cpre, total);
            if ((sn % G) == 0) {
                // First tile of a unit: wait for the unit's prefix.
                bool pok = ptx::mbar_try_wait(&ctrl->uprefix[q], (i / Q) & 1u) ||
                           ptx::mbar_wait_bounded(&ctrl->uprefix[q], (i / Q) & 1u, ptx::global_timer_ns() + long_budget);
                pok = __all_sync(kFullMask, pok);
                if (!pok && lane == 0) raise_error(a.hdr, kErrPipelineTimeout);
                run = ctrl->upre[q];
            }
            // The reduce pass left this thread's prefix within the unit.
            const T base = run + ctrl->tpre[q][sn % G][f];
#pragma unroll
            for (int c8 = 0; c8 < CHUNKS; ++c8) {
                T acc = base + cpre[c8];
#pragma unroll
                for (int e = 0; e < EPC; ++e) {
                    const T x = v[c8 * EPC + e];
                    if (INCL) {
                        acc += x;
                        v[c8 * EPC + e] = acc;
                    } else {
                        v[c8 * EPC + e] = acc;
                        acc += x;
                    }
                }
            }
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
                if ((sn % G) == G - 1) ptx::mbar_arrive(&ctrl->ufree[q]);
            }
        }
    }
}

}  // namespace gps
