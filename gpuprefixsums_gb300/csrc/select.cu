// Stream compaction (select by flags): the flag scan fused with the scatter,
// in one single-pass launch.
//
// out[0 .. count) receives, in order, the elements in[i] whose flag byte is
// non-zero; count goes to *num_selected. The structure is the chained scan's
// (decoupled lookback over 64-bit counts, as ChainedScanDecoupledLookback.cuh:
// 79-139 does for sums), with the two passes of scan_l2.cuh:
//   reduce pass  bulk-load a tile's flags (1 byte per element), turn each
//                thread's flags into a bit mask, leave every thread its mask
//                and its count-prefix within the unit in shared memory, and
//                publish the unit's count;
//   scan pass    once the previous unit's prefix is known, bulk-load the
//                tile's values, compact each thread's selected values (by
//                the reduce pass's mask) into its warp's staging slice at
//                their warp-local positions, and copy the staged run out with
//                16-byte stores at the unit prefix.
// HBM and L2 see the flags and values once each and only the selected values
// written: (sizeof(V) + 1) bytes read and p * sizeof(V) written per element
// for a selected fraction p.
//
// Warps: 0 R-loader (flags), 1 S-loader (values + flags), 2..4 lookback,
// then 4 reduce and 4 finalize warps. Every wait is bounded by the plan's
// budget.
#include "launch_util.h"
#include "scan_pipeline.cuh"

namespace gps {
namespace {

constexpr int kSelWarps = 4;                 // reduce warps = finalize warps
constexpr int kSelRole = kSelWarps * 32;     // threads per role
constexpr int kSelLookback = 3;
constexpr int kSelThreads = 32 * (2 + kSelLookback + 2 * kSelWarps);
constexpr int kSelRS = 8;   // flag stages of the reduce pass
constexpr int kSelSS = 8;   // value stages of the scan pass
constexpr int kSelQ = 6;    // units in flight
constexpr int kSelG = 4;    // tiles per unit

// 16 KB of values per tile: 4096 four-byte or 2048 eight-byte elements.
template <typename V>
struct SelShape {
    static constexpr int kTile = 16384 / static_cast<int>(sizeof(V));
    static constexpr int kItems = kTile / kSelRole;  // per thread: 128 bytes of values
    static constexpr int kEpc = 16 / static_cast<int>(sizeof(V));
    static constexpr int kChunks = kItems / kEpc;
    // A finalize warp's staging slice: its 32 rows, plus one chunk so that a
    // run can sit at the 16-byte phase of its destination.
    static constexpr int kSlice = 32 * kItems + kEpc;
};

template <typename V>
struct SelCtrl {
    uint64_t rfull[kSelRS], rfree[kSelRS];
    uint64_t sfull[kSelSS], sfree[kSelSS];
    uint64_t uknown[kSelQ], ureduced[kSelQ], uprefix[kSelQ], ufree[kSelQ];
    uint32_t r_tile[kSelRS];
    uint32_t s_tile[kSelSS];
    uint32_t unit_of[kSelQ];
    uint32_t end_seq;
    uint64_t uagg[kSelQ];
    uint64_t upre[kSelQ];
    uint32_t r_wtot[2][kSelWarps];
    uint32_t tpre[kSelQ][kSelG][kSelRole];   // count before each thread within its unit
    uint32_t tmask[kSelQ][kSelG][kSelRole];  // each thread's flags, bit e = item e
};

template <typename V>
constexpr size_t sel_smem_bytes() {
    constexpr size_t TILE = SelShape<V>::kTile;
    return kSelRS * TILE + kSelSS * TILE * sizeof(V) + kSelWarps * SelShape<V>::kSlice * sizeof(V) +
           sizeof(SelCtrl<V>);
}

struct SelArgs {
    const uint8_t* flags;
};

// Bit i set when byte i of the 4 * W bytes in w[] is non-zero.
template <int W>
__device__ __forceinline__ uint32_t nonzero_byte_mask(const uint32_t (&w)[W]) {
    uint32_t m = 0;
#pragma unroll
    for (int j = 0; j < W; ++j) {
        // 0x01 in every non-zero byte, gathered into 4 bits by one multiply.
        const uint32_t nz = __vcmpne4(w[j], 0u) & 0x01010101u;
        m |= ((nz * 0x01020408u) >> 24) << (4 * j);
    }
    return m;
}

template <typename V>
__global__ void __launch_bounds__(kSelThreads, 1) select_kernel(const ScanArgs a, const SelArgs sa) {
    using Sh = SelShape<V>;
    using D = DescTraits<uint64_t>;
    using word = D::word;
    constexpr int TILE = Sh::kTile;
    constexpr int ITEMS = Sh::kItems;
    constexpr int EPC = Sh::kEpc;
    constexpr int CHUNKS = Sh::kChunks;
    constexpr int FW = ITEMS / 4;  // flag words per thread
    constexpr uint32_t kWarpLookback = 2, kWarpReduce = 2 + kSelLookback, kWarpFinal = kWarpReduce + kSelWarps;
    constexpr int RS = kSelRS, SS = kSelSS, Q = kSelQ, G = kSelG;
    static_assert(CHUNKS == 8, "128 bytes of values per thread");
    static_assert(ITEMS <= 32, "one 32-bit mask of flags per thread");
    using Ctrl = SelCtrl<V>;

    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* rflags = smem_raw;
    V* svals = reinterpret_cast<V*>(rflags + static_cast<size_t>(RS) * TILE);
    V* ostage = svals + static_cast<size_t>(SS) * TILE;
    Ctrl* ctrl = reinterpret_cast<Ctrl*>(ostage + kSelWarps * Sh::kSlice);

    const uint32_t tid = threadIdx.x;
    const uint32_t warp = tid >> 5;
    const uint32_t lane = tid & 31u;
    const uint32_t num_units = (a.num_tiles + G - 1) / G;

    if (tid == 0) {
        for (int s = 0; s < RS; ++s) {
            ptx::mbar_init(&ctrl->rfull[s], 1);
            ptx::mbar_init(&ctrl->rfree[s], kSelWarps);
        }
        for (int s = 0; s < SS; ++s) {
            ptx::mbar_init(&ctrl->sfull[s], 1);
            ptx::mbar_init(&ctrl->sfree[s], kSelWarps);
        }
        for (int q = 0; q < Q; ++q) {
            ptx::mbar_init(&ctrl->uknown[q], 1);
            ptx::mbar_init(&ctrl->ureduced[q], kSelWarps);
            ptx::mbar_init(&ctrl->uprefix[q], 1);
            ptx::mbar_init(&ctrl->ufree[q], kSelWarps);
        }
        ctrl->end_seq = 0xFFFFFFFFu;
        ptx::fence_mbar_init();
    }
    __syncthreads();

    const uint32_t epoch = ld_volatile_u32(&a.hdr->epoch);
    const uint64_t long_budget = a.wait_budget_ns * 4 + 1000000000ull;
    auto count_of = [&](uint32_t t) -> uint32_t { return t < a.num_tiles ? tile_count<TILE>(a.n, t) : 0u; };
    auto wait1 = [&](uint64_t* bar, uint32_t ph, uint64_t b) -> bool {
        return ptx::mbar_try_wait(bar, ph) || ptx::mbar_wait_bounded(bar, ph, ptx::global_timer_ns() + b);
    };
    // A thread's flags (logical order) as a bit mask; bytes past the 16-byte
    // bulk part of a partial tile come from global memory.
    auto flag_mask = [&](const uint8_t* stage, uint32_t t, uint32_t thr) -> uint32_t {
        const uint32_t cnt = count_of(t);
        uint32_t w[FW];
        if (cnt == static_cast<uint32_t>(TILE)) {
#pragma unroll
            for (int j = 0; j < FW / 4; ++j) {
                const uint4 q4 = *reinterpret_cast<const uint4*>(stage + thr * ITEMS + 16 * j);
                w[4 * j] = q4.x;
                w[4 * j + 1] = q4.y;
                w[4 * j + 2] = q4.z;
                w[4 * j + 3] = q4.w;
            }
        } else {
            const uint32_t bulk = cnt & ~15u;
            const uint8_t* g = sa.flags + static_cast<uint64_t>(t) * TILE;
#pragma unroll
            for (int j = 0; j < FW; ++j) {
                uint32_t x = 0;
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    const uint32_t i = thr * ITEMS + 4 * j + b;
                    const uint32_t byte = i < bulk ? stage[i] : (i < cnt ? g[i] : 0u);
                    x |= (byte ? 1u : 0u) << (8 * b);
                }
                w[j] = x;
            }
        }
        return nonzero_byte_mask<FW>(w);
    };

    // ======================================================== R-loader
    if (warp == 0) {
        if (lane == 0) {
            const uint64_t pol = ptx::policy_evict_last();
            bool stop = false;
            uint32_t rn = 0;
            bool ok = true;
            for (uint32_t i = 0; ok; ++i) {
                const int q = static_cast<int>(i % Q);
                if (i >= Q && !wait1(&ctrl->ufree[q], ((i - Q) / Q) & 1u, long_budget)) break;
                uint32_t u = kTileEnd;
                if (!stop) {
                    const uint32_t raw = atomicAdd(&a.hdr->tile_counter, 1u);
                    if (raw < num_units && ld_volatile_u32(&a.hdr->error_flags) == 0)
                        u = raw;
                    else
                        stop = true;
                }
                ctrl->unit_of[q] = u;
                ptx::mbar_arrive(&ctrl->uknown[q]);
                if (u == kTileEnd) {
                    for (uint32_t m = 1; m < static_cast<uint32_t>(kSelLookback) && ok; ++m) {
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
                    const uint32_t bytes = count_of(t) & ~15u;
                    ptx::mbar_arrive_expect_tx(&ctrl->rfull[s], bytes);
                    if (bytes)
                        ptx::bulk_load_hint(rflags + static_cast<size_t>(s) * TILE,
                                            sa.flags + static_cast<uint64_t>(t) * TILE, bytes, &ctrl->rfull[s], pol);
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
                if (!wait1(&ctrl->uknown[q], (i / Q) & 1u, long_budget)) {
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
                    const uint32_t cnt = count_of(t);
                    const uint32_t vbytes = (cnt * static_cast<uint32_t>(sizeof(V))) & ~15u;
                    ptx::mbar_arrive_expect_tx(&ctrl->sfull[s], vbytes);
                    if (vbytes)
                        ptx::bulk_load_hint(svals + static_cast<size_t>(s) * TILE,
                                            static_cast<const V*>(a.in) + static_cast<uint64_t>(t) * TILE, vbytes,
                                            &ctrl->sfull[s], pol);
                }
                if (end) break;
            }
            if (!ok) raise_error(a.hdr, kErrPipelineTimeout);
        }
    }
    // ======================================================== lookback
    else if (warp < kWarpReduce) {
        word* desc = static_cast<word*>(a.desc);
        int64_t own_prev = -1;
        uint64_t own_incl = 0;
        for (uint32_t i = warp - kWarpLookback;; i += kSelLookback) {
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
            const uint64_t pre =
                u == 0 ? 0ull : lookback<uint64_t, TILE * G, false>(a, u, epoch, lane, 0ull, own_prev, own_incl);
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
            const uint64_t incl = pre + ctrl->uagg[q];
            if (lane == 0) {
                if (u != 0) D::store(desc + u, D::pack(kInclusive, epoch, incl));
                if (u == num_units - 1 && a.carry_out != nullptr) *static_cast<uint64_t*>(a.carry_out) = incl;
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
        word* desc = static_cast<word*>(a.desc);
        uint32_t unit_cnt = 0;
        for (uint32_t rn = 0;; ++rn) {
            const int s = static_cast<int>(rn % RS);
            const uint32_t i = rn / G;
            const int k = static_cast<int>(rn % G);
            const int q = static_cast<int>(i % Q);
            const bool ok = wait1(&ctrl->rfull[s], (rn / RS) & 1u, long_budget);
            const uint32_t t = ok ? ctrl->r_tile[s] : kTileEnd;
            const bool live = t != kTileEnd;
            const uint32_t m = live ? flag_mask(rflags + static_cast<size_t>(s) * TILE, t, r) : 0u;
            const uint32_t cnt = static_cast<uint32_t>(__popc(m));
            const uint32_t winc = warp_inclusive_scan(cnt, lane);
            if (lane == 31) ctrl->r_wtot[rn & 1u][rw] = winc;
            const bool stop = named_bar_or(1, kSelRole, !live || !ok);
            if (lane == 0 && live) ptx::mbar_arrive(&ctrl->rfree[s]);
            if (stop) {
                if (r == 0) {
                    if (!ok) raise_error(a.hdr, kErrPipelineTimeout);
                    *reinterpret_cast<volatile uint32_t*>(&ctrl->end_seq) = i;
                }
                break;
            }
            uint32_t wpre = 0, tot = 0;
#pragma unroll
            for (int w2 = 0; w2 < kSelWarps; ++w2) {
                const uint32_t x = ctrl->r_wtot[rn & 1u][w2];
                wpre += static_cast<uint32_t>(w2) < rw ? x : 0u;
                tot += x;
            }
            ctrl->tpre[q][k][r] = unit_cnt + wpre + (winc - cnt);
            ctrl->tmask[q][k][r] = m;
            unit_cnt += tot;
            if (k == G - 1) {
                // Each reduce warp releases its unit's prefixes and masks.
                __syncwarp();
                if (lane == 0) {
                    if (r == 0) {
                        const uint32_t u = t / G;
                        D::store(desc + u, D::pack(u == 0 ? kInclusive : kAggregate, epoch, unit_cnt));
                        ctrl->uagg[q] = unit_cnt;
                    }
                    ptx::mbar_arrive(&ctrl->ureduced[q]);
                }
                unit_cnt = 0;
            }
        }
    }
    // ======================================================== finalize
    // Thread f owns row f of each tile (ITEMS consecutive elements), so warp
    // w owns the 32 * ITEMS consecutive elements of rows 32w .. 32w + 31 and
    // compacts them into its own staging slice: each thread puts its selected
    // values at its count-prefix within the warp (from the reduce pass), then
    // the warp copies its run out with 16-byte stores (the run is staged at
    // the 16-byte phase of its destination). Only the warp synchronises, no
    // barrier between the finalize warps. The reduce pass's mask is turned
    // into register order once (the row's chunks sit rotated in registers),
    // so that every item tests a bit fixed at compile time, and each chunk's
    // first position comes from one population count: no dependent chain
    // longer than a chunk.
    else {
        const uint32_t f = tid - kWarpFinal * 32;
        const uint32_t fw = warp - kWarpFinal;
        const uint32_t rot = f & 7u;
        V* wst = ostage + fw * Sh::kSlice;  // this warp's staging slice
        uint64_t run = 0;  // the unit's output position
        for (uint32_t sn = 0;; ++sn) {
            const int s = static_cast<int>(sn % SS);
            const uint32_t i = sn / G;
            const int k = static_cast<int>(sn % G);
            const int q = static_cast<int>(i % Q);
            const bool ok = wait1(&ctrl->sfull[s], (sn / SS) & 1u, long_budget);
            const uint32_t t = ok ? ctrl->s_tile[s] : kTileEnd;
            if (__any_sync(kFullMask, t == kTileEnd)) {
                if (!ok) raise_error(a.hdr, kErrPipelineTimeout);
                break;
            }
            const V* vb = svals + static_cast<size_t>(s) * TILE;
            const uint32_t cnt = count_of(t);
            const bool full_tile = cnt == static_cast<uint32_t>(TILE);
            V v[ITEMS];
            if (full_tile) {
#pragma unroll
                for (int c8 = 0; c8 < CHUNKS; ++c8) {
                    const uint32_t c = (c8 + rot) & (CHUNKS - 1);
                    const Chunk<V> qv = *reinterpret_cast<const Chunk<V>*>(vb + f * ITEMS + c * EPC);
#pragma unroll
                    for (int e = 0; e < EPC; ++e) v[c8 * EPC + e] = qv.v[e];
                }
            } else {
                const uint32_t bulk = ((cnt * static_cast<uint32_t>(sizeof(V))) & ~15u) / sizeof(V);
                const V* g = static_cast<const V*>(a.in) + static_cast<uint64_t>(t) * TILE;
#pragma unroll
                for (int e = 0; e < ITEMS; ++e) {
                    const uint32_t li = f * ITEMS + e;
                    v[e] = li < bulk ? vb[li] : (li < cnt ? g[li] : V(0));
                }
            }
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&ctrl->sfree[s]);  // this warp is done with the stage
            if (k == 0) {
                bool pok = wait1(&ctrl->uprefix[q], (i / Q) & 1u, long_budget);
                pok = __all_sync(kFullMask, pok);
                if (!pok && lane == 0) raise_error(a.hdr, kErrPipelineTimeout);
                run = ctrl->upre[q];
            }
            const uint32_t mask = ctrl->tmask[q][k][f];  // bit e: logical item e
            const uint32_t rrot = full_tile ? rot : 0u;
            // The mask in register order: bit c8 * EPC + e is v[c8 * EPC + e].
            const uint64_t m2 = mask | (static_cast<uint64_t>(mask) << ITEMS);
            const uint32_t rm = static_cast<uint32_t>(m2 >> (rrot * EPC));
            const uint32_t warp_base = ctrl->tpre[q][k][fw * 32u];
            const uint32_t mine = ctrl->tpre[q][k][f] - warp_base;
            const uint32_t warp_cnt = __shfl_sync(kFullMask, mine + static_cast<uint32_t>(__popc(mask)), 31);
            V* out = static_cast<V*>(a.out) + run + warp_base;
            // The run's first element goes to slot o of the slice, o being its
            // destination's element phase within 16 bytes.
            const uint32_t o = static_cast<uint32_t>(reinterpret_cast<uintptr_t>(out) / sizeof(V)) & (EPC - 1);
            // The slice may still be read by this warp's previous copy-out.
            __syncwarp();
#pragma unroll
            for (int c8 = 0; c8 < CHUNKS; ++c8) {
                const uint32_t l = (c8 + rrot) & (CHUNKS - 1);
                uint32_t pos = o + mine + static_cast<uint32_t>(__popc(mask & ((1u << (l * EPC)) - 1u)));
#pragma unroll
                for (int e = 0; e < EPC; ++e) {
                    if ((rm >> (c8 * EPC + e)) & 1u) wst[pos++] = v[c8 * EPC + e];
                }
            }
            __syncwarp();
            // Copy-out: single elements up to the first 16-byte boundary, then
            // 16-byte chunks, then single elements.
            const uint32_t head = min(warp_cnt, (EPC - o) & (EPC - 1));
            const uint32_t body = (warp_cnt - head) / EPC;
            const uint32_t tail = head + body * EPC;
            if (lane < head) out[lane] = wst[o + lane];
            const Chunk<V>* src = reinterpret_cast<const Chunk<V>*>(wst + o + head);
            Chunk<V>* dst = reinterpret_cast<Chunk<V>*>(out + head);
            for (uint32_t x = lane; x < body; x += 32u) dst[x] = src[x];
            if (tail + lane < warp_cnt) out[tail + lane] = wst[o + tail + lane];
            if (k == G - 1 && lane == 0) ptx::mbar_arrive(&ctrl->ufree[q]);
        }
    }

    // Last CTA out: return the counters to zero and advance the epoch (every
    // 2^30 launches, clear the descriptors first), so that the next launch
    // needs no memset and the launch replays from a CUDA graph.
    __syncthreads();
    if (tid == 0) {
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

template <typename V>
cudaError_t launch_select_t(const ScanArgs& a, const SelArgs& sa, int num_sms, cudaStream_t stream,
                            LaunchInfo* info) {
    auto kern = select_kernel<V>;
    constexpr size_t smem = sel_smem_bytes<V>();
    static_assert(smem <= 232448, "227 KB of shared memory per CTA");
    int occ = 0;
    cudaError_t err = resident_ctas_per_sm(kern, kSelThreads, smem, &occ);
    if (err != cudaSuccess) return err;
    const uint32_t units = (a.num_tiles + kSelG - 1) / kSelG;
    const int grid = persistent_grid(units, occ, num_sms);
    if (info) *info = LaunchInfo{grid, kSelThreads, smem};
    kern<<<grid, kSelThreads, smem, stream>>>(a, sa);
    return cudaGetLastError();
}

}  // namespace

uint32_t select_tile_elems(size_t elem_size) { return elem_size == 8 ? 2048u : 4096u; }

cudaError_t launch_select(size_t elem_size, const ScanArgs& a, const uint8_t* flags, int num_sms, cudaStream_t stream,
                          LaunchInfo* info) {
    const SelArgs sa{flags};
    return elem_size == 8 ? launch_select_t<uint64_t>(a, sa, num_sms, stream, info)
                          : launch_select_t<uint32_t>(a, sa, num_sms, stream, info);
}

}  // namespace gps
