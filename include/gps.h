/*
 * gps.h -- C ABI of the GB300 device-wide prefix-scan library.
 *
 * The reference (b0nes164/GPUPrefixSums, CUDA part) exposes its scans only as
 * header-only C++ dispatcher classes that own their device buffers:
 *
 *   ChainedScanDecoupledLookbackDispatcher(uint32_t maxSize)
 *       GPUPrefixSumsCUDA/ChainedScanDecoupledLookbackDispatcher.cuh:28-34
 *   ReduceThenScanDispatcher(uint32_t maxSize)
 *       GPUPrefixSumsCUDA/ReduceThenScanDispatcher.cuh:27-32
 *   private DispatchKernelsExclusive / DispatchKernelsInclusive(uint32_t size)
 *       ChainedScanDecoupledLookbackDispatcher.cuh:177-195,
 *       ReduceThenScanDispatcher.cuh:171-187
 *
 * This header is the thin C layer those classes sit on here (see
 * include/gps_compat/ for the classes with the reference's names). A plan
 * stands for one constructed dispatcher: it fixes the algorithm, the element
 * type and the maximum size, and owns the scratch memory (tile descriptors,
 * tile sums) that the reference's constructor allocates. Unlike the reference,
 * the data buffers are the caller's: scans run on any device pointers, in place
 * or out of place, on any stream, and never write outside [0, n).
 *
 * All entry points return a gps_status; none of them synchronizes unless its
 * comment says so. Device-side waits are bounded: a wait that runs past the
 * plan's budget records a flag that gps_plan_check() reports as
 * GPS_ERR_TIMEOUT, and the kernel exits instead of hanging.
 */
#ifndef GPS_H_
#define GPS_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same type as cudaStream_t; NULL is the legacy default stream. */
typedef struct CUstream_st* gps_stream_t;

typedef enum gps_status {
    GPS_OK = 0,
    GPS_ERR_INVALID_ARGUMENT = 1,
    /* n larger than the plan's max_n. The reference prints "Error, requested
     * test size exceeds max initialized size." and returns
     * (ChainedScanDecoupledLookbackDispatcher.cuh:117-120). */
    GPS_ERR_SIZE_EXCEEDS_PLAN = 2,
    GPS_ERR_CUDA = 3,
    GPS_ERR_TIMEOUT = 4,
    GPS_ERR_UNSUPPORTED = 5,
    GPS_ERR_OUT_OF_MEMORY = 6,
    GPS_ERR_WRONG_DEVICE = 7
} gps_status;

typedef enum gps_dtype {
    GPS_DTYPE_U32 = 0, /* uint32_t, sums wrap mod 2^32 (the reference's type) */
    GPS_DTYPE_U64 = 1, /* uint64_t, sums wrap mod 2^64 */
    /* float, plain FP32 arithmetic throughout (GPS_ALGO_CSDL only). The
     * floating-point scans sum in an order fixed by n, the segments and the
     * launch configuration (gps_plan_generic_config), never by timing: two
     * runs with the same inputs and configuration give bitwise-identical
     * outputs. */
    GPS_DTYPE_F32 = 2,
    /* float in and out; each partial sum carries a TwoSum error term through
     * the thread, warp and block scans, and the value passed between lookback
     * units is FP64 (GPS_ALGO_CSDL only); repeatable like GPS_DTYPE_F32 */
    GPS_DTYPE_F32_COMPENSATED = 3,
    /* struct of four uint32_t members (16 bytes, e.g. uint4), each member
     * scanned on its own and wrapping mod 2^32 -- the reference's vec4 struct
     * scan (GPUPrefixSumsWebGPUapis/SharedShaders/csdldf_struct.wgsl:19,
     * 144-300); n counts structs; 16-byte aligned buffers (GPS_ALGO_CSDL
     * only) */
    GPS_DTYPE_U32X4 = 4
} gps_dtype;

typedef enum gps_algo {
    /* Single-pass chained scan with decoupled lookback
     * (ChainedScanDecoupledLookback.cuh:79-153). */
    GPS_ALGO_CSDL = 0,
    /* Reduce -> spine scan -> propagate, three launches
     * (ReduceThenScan.cuh:15-161, ReduceThenScanDispatcher.cuh:165-187). */
    GPS_ALGO_RTS = 1
} gps_algo;

typedef enum gps_scan_kind {
    GPS_SCAN_EXCLUSIVE = 0, /* out[i] = in[0] + ... + in[i-1], out[0] = 0 */
    GPS_SCAN_INCLUSIVE = 1  /* out[i] = in[0] + ... + in[i] */
} gps_scan_kind;

typedef struct gps_plan_s* gps_plan;

/* Version of this ABI (major*10000 + minor*100 + patch). */
int gps_version(void);

/* Text for a status code (static storage). */
const char* gps_status_string(gps_status status);

/* Text of the last error raised on this host thread ("" if none). */
const char* gps_last_error(void);

/* Creates a plan on the current device for scans of up to max_n elements
 * (max_n >= 1). Allocates and zeroes the plan's scratch memory with
 * cudaMalloc; synchronizes the device once.
 * Replaces: ChainedScanDecoupledLookbackDispatcher(uint32_t maxSize)
 * (ChainedScanDecoupledLookbackDispatcher.cuh:28-34) and
 * ReduceThenScanDispatcher(uint32_t maxSize) (ReduceThenScanDispatcher.cuh:27-32). */
gps_status gps_plan_create(gps_plan* out_plan, gps_algo algo, gps_dtype dtype, uint64_t max_n);

/* Frees the plan's scratch memory (cudaFree, which synchronizes).
 * Replaces: ~ChainedScanDecoupledLookbackDispatcher() (:158-163),
 * ~ReduceThenScanDispatcher() (ReduceThenScanDispatcher.cuh:152-156). */
gps_status gps_plan_destroy(gps_plan plan);

/* Bytes of device scratch memory the plan holds. */
gps_status gps_plan_scratch_bytes(gps_plan plan, size_t* out_bytes);

/* Prefix scan of n elements from d_in into d_out on `stream`, asynchronously.
 * d_in == d_out scans in place (as the reference always does); any other
 * overlap is rejected. Pointers must be aligned to the element size; 16-byte
 * aligned pointers take the bulk-copy (TMA) path. Only [0, n) of d_out is
 * written. n == 0 is a no-op. One plan must not be used by two scans that
 * can run at the same time (its descriptors and counters are shared).
 * Replaces: DispatchKernelsExclusive / DispatchKernelsInclusive(uint32_t size)
 * (ChainedScanDecoupledLookbackDispatcher.cuh:177-195,
 * ReduceThenScanDispatcher.cuh:171-187), which scan the dispatcher's own
 * buffer in place. */
gps_status gps_scan(gps_plan plan, gps_scan_kind kind, const void* d_in, void* d_out, uint64_t n,
                    gps_stream_t stream);

/* Batched scan: num_segments independent scans of the segments
 * [d_offsets[s], d_offsets[s+1]) of d_in (CSR offsets, uint32, num_segments + 1
 * entries, d_offsets[0] == 0 and d_offsets[num_segments] == n), in ONE launch:
 * each segment's output restarts at its first element (0 for an exclusive
 * scan). Empty segments are allowed. Any dtype on a GPS_ALGO_CSDL plan;
 * 16-byte aligned d_in and d_out; n <= 2^32 - 1; in place or out of place.
 * Asynchronous on `stream`, and capturable in a CUDA graph.
 * No counterpart in the reference: it scans one buffer per dispatch; this
 * replaces a loop of DispatchKernels{Ex,In}clusive calls, one per segment. */
gps_status gps_scan_segmented(gps_plan plan, gps_scan_kind kind, const void* d_in, void* d_out, uint64_t n,
                              const uint32_t* d_offsets, uint64_t num_segments, gps_stream_t stream);

/* Stream compaction (select by flags): copies the elements d_in[i] whose
 * flag byte d_flags[i] is non-zero, in their order, to d_out[0 .. count), and
 * writes count to *d_num_selected (uint64, device memory). One launch: the
 * flag scan is fused with the scatter, so the values and flags are read once
 * and only the selected values are written. Any GPS_ALGO_CSDL plan but a
 * struct one (GPS_DTYPE_U32X4: GPS_ERR_UNSUPPORTED); the element size is
 * the plan's (4 bytes for u32 / f32, 8 for u64). d_in and
 * d_flags 16-byte aligned, d_out aligned to the element size and not
 * overlapping them; n <= max_n. Asynchronous on `stream`; capturable.
 * No counterpart in the reference; it is the scan's next consumer (the
 * exclusive scan of the flags gives each selected element's output index). */
gps_status gps_select_flagged(gps_plan plan, const void* d_in, const uint8_t* d_flags, void* d_out, uint64_t n,
                              uint64_t* d_num_selected, gps_stream_t stream);

/* Autotuner of the batched / floating-point kernel. Times each launch
 * configuration it knows on these buffers -- tiles per lookback unit (1 or 4
 * tiles of 4096 4-byte or 2048 8-byte elements) x CTA count (one per SM, or
 * half) x threads per 128-byte row of a tile (1: each thread scans 128
 * bytes, 32 four-byte items; 2: twice the threads, 16 items each) -- and keeps
 * the fastest for every later scan of this plan of the same kind (batched or
 * plain) whose n is in the same size class (n within a factor of four). The
 * arguments are those of gps_scan_segmented (d_offsets NULL for a plain scan
 * of a floating-point or struct plan); d_in and d_out must be separate
 * buffers. On integer and struct plans every candidate's output is checked
 * against the first candidate's (a 64-bit hash computed on the device):
 * a configuration whose result differs is not taken and the call returns
 * GPS_ERR_CUDA after tuning with the others. A shape that does not fit one
 * CTA's shared memory for the element type is skipped. Without tuning a
 * size class uses one thread per row and units of 4 tiles once there are
 * two such units per SM, else 1 tile. d_out is left holding a correct
 * result. Synchronizes `stream`; not allowed while the stream is being
 * captured. The chosen configuration is returned in out_unit /
 * out_ctas_div / out_threads_per_row (any may be NULL).
 * No counterpart in the reference: its tile shape and grid are compile-time
 * constants (ChainedScanDecoupledLookbackDispatcher.cuh:13-18). */
gps_status gps_plan_autotune(gps_plan plan, gps_scan_kind kind, const void* d_in, void* d_out, uint64_t n,
                             const uint32_t* d_offsets, uint64_t num_segments, gps_stream_t stream,
                             uint32_t* out_unit, uint32_t* out_ctas_div, uint32_t* out_threads_per_row);

/* Launch configuration a batched (segmented != 0) or plain generic-kernel
 * scan of n elements would use now: tiles per unit, CTA divisor (1: one CTA
 * per SM, 2: half), threads per row (1 or 2), and whether it comes from
 * gps_plan_autotune() or gps_plan_set_generic_config(). */
gps_status gps_plan_generic_config(gps_plan plan, int segmented, uint64_t n, uint32_t* out_unit,
                                   uint32_t* out_ctas_div, uint32_t* out_threads_per_row, int* out_tuned);

/* Sets the launch configuration of a size class by hand (to restore a saved
 * tuning, or to test one configuration): unit 1 or 4, ctas_div 1 or 2,
 * threads_per_row 1 or 2. */
gps_status gps_plan_set_generic_config(gps_plan plan, int segmented, uint64_t n, uint32_t unit, uint32_t ctas_div,
                                       uint32_t threads_per_row);

/* Scan of a host array: copies h_in to the device, scans, copies the result
 * to h_out, in chunks so that the copies in both directions overlap the
 * scans; returns when h_out is complete (synchronizes `stream`). Host buffers
 * should be pinned (cudaHostAlloc / cudaHostRegister) for full speed; h_in ==
 * h_out is allowed. n may exceed the plan's max_n: the plan only bounds the
 * chunk size. Device staging memory (six chunks of up to 32 MB) is
 * allocated on first use and kept by the plan. u32 and u64 plans (others: GPS_ERR_UNSUPPORTED). */
gps_status gps_scan_host(gps_plan plan, gps_scan_kind kind, const void* h_in, void* h_out,
                         uint64_t n, gps_stream_t stream);

/* Synchronizes `stream`, then reads and clears the plan's device error
 * flags: GPS_ERR_TIMEOUT if a bounded device-side wait expired since the last
 * check (the affected output is then undefined), else GPS_OK. */
gps_status gps_plan_check(gps_plan plan, gps_stream_t stream);

/* Budget for each device-side wait of this plan's kernels, in nanoseconds
 * (default 1e9 = one second). */
gps_status gps_plan_set_wait_budget(gps_plan plan, uint64_t budget_ns);

/* Forced-stall test mode for GPS_ALGO_CSDL, in the style of the reference's
 * EmulatedDeadlocking (EmulatedDeadlocking.cuh:26-168): selected tiles
 * withhold their aggregate for up to delay_ns, and, when fallback_polls > 0,
 * a successor whose lookback sees no progress for that many polls re-reduces
 * the stalled tile's input and inserts its aggregate with a compare-and-swap.
 *   mode 0: off; mode 1: tiles with (tile % period) == 0 stall (the
 *   reference's DEADLOCK_MASK pattern with period 8); mode 2: tiles picked by
 *   a hash of (seed, tile) with probability 1/period.
 * delay_ns is at most one second. Results stay exact unless a successor's
 * wait runs past the plan's budget, which gps_plan_check() reports. */
gps_status gps_plan_set_stall(gps_plan plan, uint32_t mode, uint32_t period, uint32_t seed,
                              uint32_t delay_ns, uint32_t fallback_polls);

/* Decoupled fallback (production form of the mode above, without forced
 * stalls): a chained-scan lookback that sees no progress on a predecessor
 * for fallback_polls polls re-reduces that predecessor's input itself and
 * inserts the aggregate with a compare-and-swap, instead of waiting on. This
 * makes the scan independent of the scheduling of other CTAs, at the price
 * of re-reading a slow predecessor's input. 0 turns it off (default).
 * Integer chained-scan plans (u32, u64); batched, floating-point and select
 * launches do not use it, nor does a scan of unaligned buffers.
 * Replaces: the reference's Chained Scan with Decoupled Lookback and
 * Decoupled Fallback (README.md:9-13;
 * GPUPrefixSumsD3D12/Shaders/ChainedScanDecoupledLookbackDecoupledFallback.hlsl:81-164),
 * which the CUDA part only shows in its EmulatedDeadlocking test. */
gps_status gps_plan_set_fallback(gps_plan plan, uint32_t fallback_polls);

/* Integer scans of at most max_n elements (maximum: 64 KB of input, 16384
 * u32 or 8192 u64) run in a single CTA instead of the multi-CTA kernels.
 * Default: 64 KB on GPS_ALGO_RTS plans; 0 on GPS_ALGO_CSDL plans, whose
 * one-tile-per-CTA kernel (below) is as fast or faster at these sizes.
 * 0 sends every scan to the multi-CTA kernels. Forced-stall and fallback
 * modes always use the multi-CTA kernels. */
gps_status gps_plan_set_small_max(gps_plan plan, uint64_t max_n);

/* Integer scans on a GPS_ALGO_CSDL plan above the one-CTA size and of at
 * most max_n elements (default: 64 MB of input, 2^24 u32 or 2^23 u64) run
 * as one 16 KB tile per CTA -- a single-pass chained scan without
 * the persistent kernel's pipeline, whose latency dominates at these sizes;
 * larger ones run on the persistent L2-buffered kernel. 0 sends them all to
 * the persistent kernel. Forced-stall and fallback modes always use the
 * persistent kernel. The kernel takes its tile ids from the block index and
 * relies on the hardware starting lower-numbered blocks first, as CUB's
 * decoupled lookback does; its waits are bounded all the same. */
gps_status gps_plan_set_mid_max(gps_plan plan, uint64_t max_n);

/* Lookback statistics gathered while forced-stall mode is on. Synchronizes
 * `stream`. */
typedef struct gps_lookback_stats {
    uint64_t polls;     /* lookback windows that had to be re-read */
    uint64_t fallbacks; /* stalled predecessors re-reduced by a successor */
    uint64_t inserts;   /* re-reduced aggregates that won the compare-and-swap */
    uint64_t stalls;    /* tiles that stalled */
} gps_lookback_stats;
gps_status gps_plan_stats(gps_plan plan, gps_stream_t stream, gps_lookback_stats* out_stats);

/* Kernel geometry of the plan (for tools and tests): elements per tile of the
 * main scan kernel, its grid size for a scan of n elements, and the number of
 * kernel launches one gps_scan of n elements makes. */
gps_status gps_plan_geometry(gps_plan plan, uint64_t n, uint32_t* tile_elems, uint32_t* grid,
                             uint32_t* launches);

/* Largest n gps_scan_u32_noalloc() accepts: 2^28 elements. */
#define GPS_NOALLOC_MAX_N (1ull << 28)

/* Chained scan of n uint32 elements that allocates nothing -- for callers
 * that may not call cudaMalloc (a fixed device-memory budget set by the host
 * application, a context where the allocator must not be entered, or a
 * latency-critical path that cannot pay for cudaMalloc's synchronisation).
 * No counterpart in the reference: its dispatchers always allocate in their
 * constructors.
 *
 * The scratch memory (workspace header and tile descriptors, about 513 KB)
 * is a fixed array of the library that every GPU which loads the library
 * holds until the process exits. Same semantics as gps_scan() on a GPS_ALGO_CSDL
 * / GPS_DTYPE_U32 plan, without a plan: in place or out of place, nothing
 * written outside [0, n), asynchronous on `stream`. n above
 * GPS_NOALLOC_MAX_N returns GPS_ERR_SIZE_EXCEEDS_PLAN.
 *
 * The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current, and sets up the launch
 * attributes of all four kernels the call can launch (exclusive and
 * inclusive, 16-byte-aligned and other buffers); make that first call before
 * any stream capture starts. The set-up belongs to the CUDA context it was
 * made in: after cudaDeviceReset(), or with another driver context current
 * on the device, the next call makes it again, and that call too should come
 * before any capture.
 * Every call clears the part of the array it uses with cudaMemsetAsync on
 * `stream`, because the array keeps what the previous call left. All calls
 * share the one array: two calls that can run at the same time on the GPU
 * (different streams, different host threads) race and give wrong results.
 * Device-side waits are bounded (one second each) but this entry point has
 * no plan to report a timeout through: a call whose wait ran out returns
 * GPS_OK with an undefined output, and the next call clears the record. */
gps_status gps_scan_u32_noalloc(gps_scan_kind kind, const void* d_in, void* d_out, uint64_t n,
                                gps_stream_t stream);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* GPS_H_ */
