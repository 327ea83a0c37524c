#!/usr/bin/env python3
"""Benchmark of the device-wide scan on GB300.

Workload (one step): exclusive prefix scan of n = 2^28 uint32 values
(uniform [0, 255], seeded, synthetic), out of place, by the single-pass
chained scan (GPS_ALGO_CSDL) through the C ABI (gps_scan). Inputs and outputs
are 1 GiB each, larger than the 129 MB L2, so no flush is needed between
steps.

Reported (one JSON line on rank 0):
  value        whole-job GB/s of algorithmic traffic (8 bytes per element:
               one read, one write), device-resident data;
  roofline     the scan kernel's achieved GB/s against the measured HBM copy
               bandwidth; DRAM traffic per launch from the committed ncu
               summary;
  e2e          the same metric through gps_scan_host with pinned host
               buffers (host->device and device->host copies timed);
  compare      D2D copy of the same bytes (the 100% line), CUB DeviceScan and
               the reduce-then-scan path on the same buffers;
  cpu_baseline the oracle's serial scan on one host core;
  sweep        the chained scan by size (2^10 .. 2^28 u32) and u64 at 2^27;
  batched      4096 independent u32 exclusive scans, lengths log-uniform in
               [1, 2^20] (seeded), CSR offsets: one autotuned launch replayed
               from a CUDA graph against a graph of one plain scan per segment
               (identical output checked), speed-up and GB/s;
  fp32         inclusive scans of 2^26 floats, N(0,1) and mixed magnitude
               (|x| log-uniform in [1e-8, 1e8], random sign): plain and
               compensated FP32 throughput and errors against a float64 scan;
  mixed        10,000 scans, lengths Zipf(1.2) in [32, 2^22], dtype per scan
               from {u32, u64, compensated f32}, plus a 2^28-element u32
               Bernoulli(0.3) flag scan, all in one CUDA graph;
  select       stream compaction of 2^28 u32 values by Bernoulli(0.3) flag
               bytes in one launch, beside CUB's DeviceSelect::Flagged.
With --impl reference the line times the reference's own algorithm on the
host instead (the oracle's multi-threaded restatement, all host threads): the
reference ships no CPU scan of its own.

Multi-GPU (torchrun): every rank scans its own 2^28 elements (replicas,
weak scaling); the slowest rank's time is used.
"""
from __future__ import annotations

import argparse
import ctypes
import datetime
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PROFILE_TRAFFIC = os.path.join(ROOT, "profiles", "scan_l2_kernel_u32_exclusive_2pow28.md")
METRIC = "scan GB/s (u32 exclusive, n=2^28, chained scan), % of D2D-copy roofline"


def parse_args():
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=4000)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--n", type=int, default=1 << 28, help="elements per scan")
    p.add_argument("--algo", choices=["csdl", "rts"], default="csdl")
    p.add_argument("--no-compare", action="store_true",
                   help="only the timed scans (for profiling): no copy/CUB/RTS/e2e/CPU legs")
    p.add_argument("--no-extras", action="store_true", help="skip the batched, fp32 and mixed workloads")
    p.add_argument("--profile-case", choices=["batched", "f32c", "select", "struct", "mid", "f32c_batched",
                                              "u64_batched"], default=None,
                   help="launch one small case three times and exit (ncu captures): 1024 of the batched "
                        "workload's segments, 2^26 compensated-f32 elements, a select of 2^26 u32 by "
                        "Bernoulli(0.3) flags, an inclusive scan of 2^24 structs of four u32, an "
                        "exclusive u32 scan of 2^20 elements (the one-tile-per-CTA kernel), or the first "
                        "1000 compensated-f32 / u64 segments of the mixed workload")
    p.add_argument("--e2e-steps", type=int, default=8)
    p.add_argument("--clock-soak-s", type=float, default=1.0,
                   help="seconds of untimed steps sampled for clocks right before the timed region")
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    return p.parse_args()


# ----------------------------------------------------------------- helpers
INPUT_SEED = 2028


def workload_config(args, world):
    """The workload both arms time, described identically: the same n, the
    same values (numpy default_rng(INPUT_SEED + rank), uniform [0, 255])."""
    return {"workload": f"u32 exclusive scan of n={args.n} elements, out of place, values uniform [0,255] from "
                        f"numpy default_rng({INPUT_SEED} + rank)",
            "n": args.n, "seed": INPUT_SEED, "parallelism": f"replicas x{world}",
            "l2": "inputs and outputs of 1 GiB each exceed the 129 MB L2; no flush needed"}


def workload_input(args, rank):
    """The seeded input of one rank, on the host (uint32)."""
    import numpy as np
    return np.random.default_rng(INPUT_SEED + rank).integers(0, 256, size=args.n, dtype=np.uint32)


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        if d.get("hbm_gbs"):
            return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic_per_elem():
    """DRAM bytes per element of the scan kernel from the committed ncu
    summary (line 'dram_bytes_per_element: X'), or None."""
    if not os.path.exists(PROFILE_TRAFFIC):
        return None, None
    with open(PROFILE_TRAFFIC) as f:
        for line in f:
            if line.startswith("dram_bytes_per_element:"):
                return float(line.split(":", 1)[1]), os.path.relpath(PROFILE_TRAFFIC, ROOT)
    return None, None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 50 ms. The timed
    region of a short run lasts milliseconds, so the window read back starts
    with a soak of back-to-back untimed steps (about a second) just before it
    and ends with it: the samples see the same load as the timed steps."""
    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    REASONS = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, device_index):
        self.proc = None
        self.path = None
        try:
            import torch
            uuid = str(torch.cuda.get_device_properties(device_index).uuid)
            ident = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
            fd, self.path = tempfile.mkstemp(prefix="gps_clocks_", suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "50", "-i", ident], stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self, t_soak, t0, t1):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "note": "nvidia-smi unavailable"}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        self.out.close()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 10:
                    continue
                try:
                    ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                    rows.append((ts, float(parts[2]), float(parts[3]), parts[6:10]))
                except ValueError:
                    continue
        os.unlink(self.path)
        window = [r for r in rows if t_soak <= r[0] <= t1 + 0.05]
        if not window:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "note": "no samples"}
        reasons = sorted({self.REASONS[i] for r in window for i, v in enumerate(r[3]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[1] for r in window), "sm_max_mhz": max(r[2] for r in window),
                "reasons": reasons, "samples": len(window),
                "samples_in_timed_region": sum(1 for r in window if t0 - 0.05 <= r[0] <= t1 + 0.05),
                "window_s": round(t1 - t_soak, 3),
                "window": "soak of back-to-back untimed steps just before the timed region, then the timed region"}


def max_over_ranks(value, dist=None, device="cuda"):
    """The slowest rank's figure (times are maxed over ranks); the value
    itself on a single process."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def time_loop(fn, steps, stream):
    import torch
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(steps):
        fn()
    stop.record(stream)
    stop.synchronize()
    return start.elapsed_time(stop) / steps  # ms per call


# ------------------------------------------------------------- reference
def run_reference(args, world, rank):
    """The reference's algorithm on the host cores: the oracle's three-phase
    (reduce, spine, propagate) restatement on every host thread."""
    if rank != 0:
        return
    import numpy as np

    import oracle
    threads = os.cpu_count() or 1
    full = workload_input(args, rank)
    out = np.empty_like(full)
    t = time.perf_counter()
    oracle.scan_mt(full, out=out, inclusive=False, threads=threads)
    t_full = time.perf_counter() - t
    # Bounded sample per step: the whole run stays within about two minutes,
    # but never below 2^25 elements (128 MB, beyond the host's last-level cache).
    per_step = 100.0 / max(1, args.steps + args.warmup)
    sample = int(min(args.n, max(1 << 25, args.n * per_step / max(t_full, 1e-9))))
    x = full[:sample]
    y = out[:sample]
    for _ in range(args.warmup):
        oracle.scan_mt(x, out=y, inclusive=False, threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.scan_mt(x, out=y, inclusive=False, threads=threads)
    dt = (time.perf_counter() - t0) / args.steps
    gbs = sample * 8 / dt / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(gbs, 3), "unit": "GB/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": workload_config(args, world),
        "cpu_baseline": {"value": round(gbs, 3), "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} of the {args.n} elements per step (3-phase reduce-then-scan "
                                   f"restated in oracle/scan_oracle.c, {threads} threads)"},
        "e2e": {"value": round(gbs, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------- workload extras
def graph_of(fn, stream):
    """Captures fn (which launches on `stream`) in a CUDA graph; returns a
    callable that replays it on `stream`."""
    import torch
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        fn()  # warm-up outside the capture (first-use setup)
        stream.synchronize()
        with torch.cuda.graph(g, stream=stream):
            fn()
    stream.synchronize()

    def replay():
        with torch.cuda.stream(stream):  # replay() launches on the current stream
            g.replay()
    replay.graph = g
    return replay


def log_uniform_lengths(count, hi, seed):
    import numpy as np
    rng = np.random.default_rng(seed)
    return np.floor(np.exp(rng.uniform(0.0, np.log(float(hi)), size=count))).astype(np.int64)


def zipf_lengths(count, s, lo, hi, seed):
    """Continuous Zipf(s) (density ~ x^-s) truncated to [lo, hi], floored:
    inverse CDF of a seeded uniform."""
    import numpy as np
    rng = np.random.default_rng(seed)
    u = rng.uniform(0.0, 1.0, size=count)
    a, b = lo ** (1.0 - s), hi ** (1.0 - s)
    x = (a - u * (a - b)) ** (1.0 / (1.0 - s))
    return np.clip(np.floor(x), lo, hi).astype(np.int64)


def run_batched(stream, copy_gbs, reps=20):
    """4096 u32 exclusive scans in one launch vs one plain launch per scan."""
    import numpy as np
    import torch

    from gpuprefixsums_gb300 import Plan
    lengths = log_uniform_lengths(4096, 2 ** 20, seed=3)
    offs = np.concatenate([[0], np.cumsum(lengths)]).astype(np.uint32)
    n = int(offs[-1])
    gen = torch.Generator(device="cuda").manual_seed(4096)
    x = torch.randint(0, 256, (n,), dtype=torch.int32, device="cuda", generator=gen)
    d_off = torch.from_numpy(offs.view(np.int32)).cuda()
    out_b, out_l = torch.empty_like(x), torch.empty_like(x)
    segs = [(int(offs[i]), int(offs[i + 1])) for i in range(len(lengths)) if offs[i + 1] > offs[i]]
    with Plan("csdl", "u32", max_n=n) as plan:
        tuned = plan.autotune(x, d_off, out=out_b, stream=stream)
        gb = graph_of(lambda: plan.scan_segmented(x, d_off, out=out_b, stream=stream), stream)
        xp, op = x.data_ptr(), out_l.data_ptr()

        def looped():
            for b, e in segs:
                plan.scan_ptr(xp + 4 * b, op + 4 * b, e - b, stream=stream)
        gl = graph_of(looped, stream)
        for _ in range(3):
            gb()
        ms_b = time_loop(gb, reps, stream)
        gl()
        ms_l = time_loop(gl, 3, stream)
        looped()
        ms_e = time_loop(looped, 2, stream)
        plan.check(stream)
        same = bool(torch.equal(out_b, out_l))
    if not same:
        raise SystemExit("bench: batched and looped scans differ; refusing to report a number")
    alg = n * 8 + 4 * len(offs)
    gbs = alg / (ms_b * 1e-3) / 1e9
    return {"workload": "4096 u32 exclusive scans, lengths floor(log-uniform[1, 2^20]) seed 3, values uniform "
                        "[0,255], CSR uint32 offsets; batched = 1 launch replayed from a CUDA graph",
            "elements": n, "segments": len(lengths), "ms_batched": round(ms_b, 4),
            "ms_looped_graph": round(ms_l, 3), "ms_looped_eager": round(ms_e, 3),
            "speedup_vs_looped_graph": round(ms_l / ms_b, 2), "speedup_vs_looped_eager": round(ms_e / ms_b, 2),
            "gbs": round(gbs, 2), "pct_of_copy": round(100.0 * gbs / copy_gbs, 2) if copy_gbs else None,
            "identical_to_looped": same, "autotuned": tuned, "launches_per_step": 1}


def run_select(stream, copy_gbs, reps=20):
    """Stream compaction of 2^28 u32 values by Bernoulli(0.3) flag bytes:
    the fused select against CUB's DeviceSelect::Flagged on the same data."""
    import torch

    from gpuprefixsums_gb300 import Plan
    from gpuprefixsums_gb300 import build as gbuild
    n = 1 << 28
    gen = torch.Generator(device="cuda").manual_seed(303)
    x = torch.randint(-2 ** 31, 2 ** 31 - 1, (n,), dtype=torch.int32, device="cuda", generator=gen)
    fl = (torch.rand(n, device="cuda", generator=gen) < 0.3).to(torch.uint8)
    out = torch.empty_like(x)
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    res = {"workload": "select 2^28 u32 by Bernoulli(0.3) flag bytes (fused flag scan + scatter, 1 launch)"}
    with Plan("csdl", "u32", max_n=n) as plan:
        step = lambda: plan.select(x, fl, out=out, num_selected=cnt, stream=stream)  # noqa: E731
        for _ in range(3):
            step()
        ms = time_loop(step, reps, stream)
        plan.check(stream)
    c = int(cnt.item())
    if not torch.equal(out[:c], torch.masked_select(x, fl.bool())):
        raise SystemExit("bench: select result is wrong; refusing to report a number")
    alg = n * 5 + c * 4
    res.update({"selected": c, "ms": round(ms, 4), "gbs": round(alg / (ms * 1e-3) / 1e9, 2),
                "elements_per_s": round(n / (ms * 1e-3), 1),
                "pct_of_copy": round(100.0 * alg / (ms * 1e-3) / 1e9 / copy_gbs, 2) if copy_gbs else None,
                "bytes_per_element": round(alg / n, 3)})
    try:
        cub = ctypes.CDLL(gbuild.build_cub_compare())
        cub.gps_cub_select_u32.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_uint64, ctypes.c_void_p,
                                                                     ctypes.POINTER(ctypes.c_size_t), ctypes.c_void_p]
        tb = ctypes.c_size_t(0)
        cub.gps_cub_select_u32(x.data_ptr(), fl.data_ptr(), out.data_ptr(), cnt.data_ptr(), n, None, ctypes.byref(tb),
                               None)
        temp = torch.empty(max(1, tb.value), dtype=torch.uint8, device="cuda")
        sp = ctypes.c_void_p(stream.cuda_stream)
        cub_call = lambda: cub.gps_cub_select_u32(x.data_ptr(), fl.data_ptr(), out.data_ptr(),  # noqa: E731
                                                  cnt.data_ptr(), n, temp.data_ptr(), ctypes.byref(tb), sp)
        for _ in range(3):
            cub_call()
        cub_ms = time_loop(cub_call, reps, stream)
        res["cub_select_ms"] = round(cub_ms, 4)
        res["ours_vs_cub"] = round(cub_ms / ms, 3)
    except Exception as e:  # comparison only
        res["cub_error"] = str(e)[:200]
    return res


def run_struct(stream, copy_gbs, reps=20):
    """Struct scan: inclusive scan of 2^26 structs of four u32 members (1 GiB
    in, 1 GiB out), each member on its own; against CUB's DeviceScan with a
    member-wise sum on the same data."""
    import torch

    from gpuprefixsums_gb300 import Plan
    from gpuprefixsums_gb300 import build as gbuild
    n = 1 << 26
    gen = torch.Generator(device="cuda").manual_seed(404)
    x = torch.randint(-2 ** 31, 2 ** 31 - 1, (n, 4), dtype=torch.int32, device="cuda", generator=gen)
    out = torch.empty_like(x)
    res = {"workload": "inclusive struct scan of 2^26 x (4 x u32) = 1 GiB (member-wise, one launch)"}
    with Plan("csdl", "u32x4", max_n=n) as plan:
        step = lambda: plan.scan(x, out, inclusive=True, stream=stream)  # noqa: E731
        for _ in range(3):
            step()
        ms = time_loop(step, reps, stream)
        plan.check(stream)
    if not (torch.equal(out[1:] - out[:-1], x[1:]) and torch.equal(out[0], x[0])):
        raise SystemExit("bench: struct scan result is wrong; refusing to report a number")
    gbs = n * 32 / (ms * 1e-3) / 1e9
    res.update({"ms": round(ms, 4), "gbs": round(gbs, 2), "structs_per_s": round(n / (ms * 1e-3), 1),
                "pct_of_copy": round(100.0 * gbs / copy_gbs, 2) if copy_gbs else None})
    try:
        cub = ctypes.CDLL(gbuild.build_cub_compare())
        cub.gps_cub_scan_u32x4.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                                           ctypes.POINTER(ctypes.c_size_t), ctypes.c_void_p]
        tb = ctypes.c_size_t(0)
        cub.gps_cub_scan_u32x4(x.data_ptr(), out.data_ptr(), n, None, ctypes.byref(tb), None)
        temp = torch.empty(max(1, tb.value), dtype=torch.uint8, device="cuda")
        sp = ctypes.c_void_p(stream.cuda_stream)
        cub_call = lambda: cub.gps_cub_scan_u32x4(x.data_ptr(), out.data_ptr(), n, temp.data_ptr(),  # noqa: E731
                                                  ctypes.byref(tb), sp)
        for _ in range(3):
            cub_call()
        cub_ms = time_loop(cub_call, reps, stream)
        res["cub_ms"] = round(cub_ms, 4)
        res["ours_vs_cub"] = round(cub_ms / ms, 3)
    except Exception as e:  # comparison only
        res["cub_error"] = str(e)[:200]
    return res


def graph_us(fn, stream, k):
    """GPU time per call of fn (which launches on `stream`): k calls captured
    in one CUDA graph, the graph replayed 5 times, CUDA events around the
    replays -- the host's launch rate does not enter, unlike a Python loop of
    launches at small sizes."""
    import torch
    with torch.cuda.stream(stream):
        for _ in range(3):
            fn()
        stream.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            for _ in range(k):
                fn()
        g.replay()
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for _ in range(5):
            g.replay()
        stop.record(stream)
        stop.synchronize()
    return start.elapsed_time(stop) * 1e3 / (5 * k)


def run_sweep(stream, d_in, d_out):
    """Config-2 sizes: u32 exclusive chained scan at n = 2^10 .. 2^28 (every
    second power of two) on the benchmark's buffers, beside CUB DeviceScan on
    the same buffers, and u64 at n = 2^27. GPU time per scan from CUDA-graph
    replay. Inputs below about 2^24 elements stay in L2 between launches.
    The plan's defaults pick the kernel: one tile per CTA up to 64 MB, the
    persistent L2-buffered kernel above."""
    import torch

    from gpuprefixsums_gb300 import Plan
    from gpuprefixsums_gb300 import build as gbuild
    res = {"workload": "u32 exclusive chained scan by size (L2-resident below ~2^24; GPU time per scan from "
                       "CUDA-graph replay), u64 exclusive at 2^27",
           "u32": {}}
    cub = None
    try:
        cub = ctypes.CDLL(gbuild.build_cub_compare())
        cub.gps_cub_scan_u32.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                         ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t), ctypes.c_void_p]
        tb = ctypes.c_size_t(0)
        cub.gps_cub_scan_u32(0, d_in.data_ptr(), d_out.data_ptr(), d_in.numel(), None, ctypes.byref(tb), None)
        temp = torch.empty(max(1, tb.value), dtype=torch.uint8, device="cuda")
    except Exception as e:  # comparison only
        res["cub_error"] = str(e)[:200]
    sp = ctypes.c_void_p(stream.cuda_stream)
    with Plan("csdl", "u32", max_n=d_in.numel()) as plan:
        for k in range(10, 29, 2):
            n = 1 << k
            reps = max(4, min(50, (1 << 26) // n))
            us = graph_us(lambda: plan.scan(d_in, d_out, n=n, stream=stream), stream, reps)
            row = {"gbs": round(n * 8 / (us * 1e-6) / 1e9, 2), "us": round(us, 2)}
            if cub is not None:
                row["cub_us"] = round(graph_us(lambda: cub.gps_cub_scan_u32(0, d_in.data_ptr(), d_out.data_ptr(), n,
                                                                            temp.data_ptr(), ctypes.byref(tb), sp),
                                               stream, reps), 2)
            res["u32"][f"2^{k}"] = row
        plan.check(stream)
    n64 = 1 << 27
    x64, o64 = d_in.view(torch.int64)[:n64], d_out.view(torch.int64)[:n64]
    with Plan("csdl", "u64", max_n=n64) as plan:
        step = lambda: plan.scan(x64, o64, stream=stream)  # noqa: E731
        for _ in range(3):
            step()
        ms = time_loop(step, 50, stream)
        plan.check(stream)
    res["u64_2^27_gbs"] = round(n64 * 16 / (ms * 1e-3) / 1e9, 2)
    return res


def fp_errors_vs_f64(got, ref):
    """max / median relative prefix error (nonzero reference prefixes) and
    relative error of the final sum, against a float64 scan."""
    import torch
    g = got.double()
    nz = ref != 0
    rel = (g[nz] - ref[nz]).abs() / ref[nz].abs()
    fin = float(((g[-1] - ref[-1]).abs() / ref[-1].abs()).item()) if float(ref[-1]) != 0 else None
    return {"max_rel": float(rel.max().item()), "median_rel": float(torch.median(rel).item()),
            "final_sum_rel": fin}


def run_fp32(stream, reps=20):
    import torch

    from gpuprefixsums_gb300 import Plan
    n = 1 << 26
    gen = torch.Generator(device="cuda").manual_seed(26)
    sets = {"normal": torch.randn(n, device="cuda", generator=gen)}
    mag = torch.exp(torch.empty(n, device="cuda", dtype=torch.float64).uniform_(
        float(torch.log(torch.tensor(1e-8, dtype=torch.float64))),
        float(torch.log(torch.tensor(1e8, dtype=torch.float64))), generator=gen))
    sign = torch.where(torch.rand(n, device="cuda", generator=gen) < 0.5, -1.0, 1.0).double()
    sets["mixed"] = (mag * sign).float()
    del mag, sign
    res = {"workload": "inclusive scans of 2^26 float32, N(0,1) and |x| log-uniform [1e-8,1e8] with random sign; "
                       "errors against torch.cumsum in float64 on the same inputs",
           "n": n}
    out = torch.empty(n, device="cuda")
    for name, x in sets.items():
        ref = torch.cumsum(x.double(), 0)
        row = {}
        for dt in ("f32", "f32c"):
            with Plan("csdl", dt, max_n=n) as plan:
                step = lambda: plan.scan(x, out, inclusive=True, stream=stream)  # noqa: E731
                for _ in range(3):
                    step()
                ms = time_loop(step, reps, stream)
                plan.check(stream)
                row[dt] = {"gbs": round(n * 8 / (ms * 1e-3) / 1e9, 2), "ms": round(ms, 4),
                           **fp_errors_vs_f64(out, ref)}
        row["compensated_cost_pct"] = round(100.0 * (row["f32"]["gbs"] / row["f32c"]["gbs"] - 1.0), 1)
        res[name] = row
    return res


def run_mixed(stream, copy_gbs, reps=5):
    """Config of 10,000 mixed-dtype scans plus a 2^28 flag scan, one graph."""
    import numpy as np
    import torch

    from gpuprefixsums_gb300 import Plan
    count = 10_000
    lengths = zipf_lengths(count, 1.2, 32, 2 ** 22, seed=5)
    kinds = np.random.default_rng(55).integers(0, 3, size=count)  # 0 u32, 1 u64, 2 f32c
    gen = torch.Generator(device="cuda").manual_seed(5)
    groups = {}
    for k, (name, tdt) in enumerate((("u32", torch.int32), ("u64", torch.int64), ("f32c", torch.float32))):
        ls = lengths[kinds == k]
        offs = np.concatenate([[0], np.cumsum(ls)]).astype(np.uint32)
        m = int(offs[-1])
        if name == "u32":
            x = torch.randint(0, 256, (m,), dtype=tdt, device="cuda", generator=gen)
        elif name == "u64":
            x = torch.randint(-2 ** 63, 2 ** 63 - 1, (m,), dtype=tdt, device="cuda", generator=gen)
        else:
            x = torch.randn(m, device="cuda", generator=gen)
        groups[name] = {"x": x, "out": torch.empty_like(x), "offs": torch.from_numpy(offs.view(np.int32)).cuda(),
                        "offs_host": offs, "plan": Plan("csdl", name, max_n=m), "m": m, "scans": len(ls)}
    nf = 1 << 28
    flags = (torch.rand(nf, device="cuda", generator=gen) < 0.3).to(torch.int32)
    fout = torch.empty_like(flags)
    fplan = Plan("csdl", "u32", max_n=nf)
    for g in groups.values():
        g["plan"].autotune(g["x"], g["offs"], out=g["out"], stream=stream)

    def batch():
        for g in groups.values():
            g["plan"].scan_segmented(g["x"], g["offs"], out=g["out"], stream=stream)
        fplan.scan(flags, fout, inclusive=False, stream=stream)
    graph = graph_of(batch, stream)
    graph()
    ms = time_loop(graph, reps, stream)
    for g in groups.values():
        g["plan"].check(stream)
    fplan.check(stream)
    # Exactness of the integer groups and the flag scan (difference property),
    # error of the float group against per-segment float64 scans.
    ok = True
    ok &= bool((groups["f32c"]["out"][torch.from_numpy(groups["f32c"]["offs_host"][:-1].astype(np.int64)).cuda()]
                == 0).all())
    for name in ("u32", "u64"):
        g = groups[name]
        o, x, offs = g["out"], g["x"], g["offs_host"]
        if name == "u32":
            d = (o[1:].to(torch.int64) - o[:-1].to(torch.int64)) & 0xFFFFFFFF
            want = x[:-1].to(torch.int64)
        else:
            d, want = o[1:] - o[:-1], x[:-1]
        starts = torch.from_numpy(offs[1:-1].astype(np.int64)).cuda()
        inner = torch.ones(g["m"] - 1, dtype=torch.bool, device="cuda")
        inner[starts[starts > 0] - 1] = False
        ok &= bool(torch.equal(d[inner], want[inner])) and bool((o[starts.clamp(max=g["m"] - 1)] == 0).all())
    d = fout[1:] - fout[:-1]
    ok &= int(fout[0]) == 0 and bool(torch.equal(d, flags[:-1]))
    if not ok:
        raise SystemExit("bench: mixed batch result is wrong; refusing to report a number")
    g = groups["f32c"]
    worst, med = 0.0, []
    offs = g["offs_host"]
    for i in range(len(offs) - 1):
        b, e = int(offs[i]), int(offs[i + 1])
        if e > b:
            incl = torch.cumsum(g["x"][b:e].double(), 0)
            err = fp_errors_vs_f64(g["out"][b + 1:e], incl[:-1])  # exclusive: out[b] == 0 is checked above
            worst = max(worst, err["max_rel"])
            med.append(err["median_rel"])
    elems = sum(g["m"] for g in groups.values()) + nf
    alg = sum(g["m"] * g["x"].element_size() * 2 + 4 * len(g["offs_host"]) for g in groups.values()) + nf * 8
    gbs = alg / (ms * 1e-3) / 1e9
    res = {"workload": "10,000 scans, lengths Zipf(1.2) floored in [32, 2^22] seed 5, dtype per scan uniform over "
                       "{u32 [0,255], u64 full range, compensated f32 N(0,1)}, batched per dtype; plus an exclusive "
                       "scan of 2^28 u32 Bernoulli(0.3) flags; 4 launches in one CUDA graph",
           "scans": {k: g["scans"] for k, g in groups.items()}, "elements": elems, "ms": round(ms, 3),
           "elements_per_s": round(elems / (ms * 1e-3), 1), "gbs": round(gbs, 2),
           "pct_of_copy": round(100.0 * gbs / copy_gbs, 2) if copy_gbs else None,
           "f32c_max_rel_err": worst, "f32c_median_rel_err": float(np.median(med)), "exact_integer_groups": ok,
           "launches_per_step": 4}
    for g in groups.values():
        g["plan"].close()
    fplan.close()
    return res


# ------------------------------------------------------------------ ours
def run_ours(args, world, rank, local):
    import numpy as np
    import torch

    from gpuprefixsums_gb300 import Plan
    from gpuprefixsums_gb300 import build as gbuild

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    n = args.n
    stream = torch.cuda.Stream()
    h_in = torch.from_numpy(workload_input(args, rank).view(np.int32)).pin_memory()
    with torch.cuda.stream(stream):
        d_in = h_in.to("cuda", non_blocking=True)
        d_out = torch.empty_like(d_in)
    stream.synchronize()
    plan = Plan(args.algo, "u32", max_n=n)
    launches = plan.geometry(n)["launches"]
    step = lambda: plan.scan(d_in, d_out, inclusive=False, stream=stream)  # noqa: E731

    # Result check before timing (no oracle here): d_out[0] == 0 and
    # d_out[i+1] - d_out[i] == d_in[i] mod 2^32.
    step()
    stream.synchronize()
    plan.check(stream)
    diff = (d_out[1:].to(torch.int64) - d_out[:-1].to(torch.int64)) & 0xFFFFFFFF
    ok = int(d_out[0]) == 0 and torch.equal(diff, d_in[:-1].to(torch.int64))
    del diff
    if not ok:
        raise SystemExit("bench: scan result is wrong; refusing to report a number")

    for _ in range(args.warmup):
        step()
    stream.synchronize()
    sampler = ClockSampler(local)
    time.sleep(0.4)
    # Clock soak: about a second of the same untimed steps, sampled together
    # with the timed region that follows at once.
    t_soak = time.time()
    while time.time() - t_soak < args.clock_soak_s:
        for _ in range(64):
            step()
        stream.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.time()
    ms = time_loop(step, args.steps, stream)
    torch.cuda.synchronize()
    t1 = time.time()
    if dist:
        dist.barrier()
    clocks = sampler.stop(t_soak, t0, t1)
    plan.check(stream)
    ms = max_over_ranks(ms, dist)
    alg_bytes = n * 8
    value = world * alg_bytes / (ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak()
    kernel_gbs = alg_bytes / (ms / launches * 1e-3) / 1e9 if launches == 1 else None

    compare, e2e, cpu, extras = {}, None, None, {}
    if not args.no_compare:
        reps = 30

        def copy_on_stream():
            with torch.cuda.stream(stream):
                d_out.copy_(d_in)

        for _ in range(3):
            copy_on_stream()
        copy_ms = time_loop(copy_on_stream, reps, stream)
        compare["d2d_copy_gbs"] = round(alg_bytes / (copy_ms * 1e-3) / 1e9, 2)
        compare["pct_of_copy"] = round(100.0 * copy_ms / ms, 2)
        try:
            cub = ctypes.CDLL(gbuild.build_cub_compare())
            cub.gps_cub_scan_u32.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                             ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t), ctypes.c_void_p]
            tb = ctypes.c_size_t(0)
            cub.gps_cub_scan_u32(0, d_in.data_ptr(), d_out.data_ptr(), n, None, ctypes.byref(tb), None)
            temp = torch.empty(max(1, tb.value), dtype=torch.uint8, device="cuda")
            sp = ctypes.c_void_p(stream.cuda_stream)
            cub_call = lambda: cub.gps_cub_scan_u32(0, d_in.data_ptr(), d_out.data_ptr(), n,  # noqa: E731
                                                    temp.data_ptr(), ctypes.byref(tb), sp)
            for _ in range(3):
                cub_call()
            cub_ms = time_loop(cub_call, reps, stream)
            compare["cub_exclusive_gbs"] = round(alg_bytes / (cub_ms * 1e-3) / 1e9, 2)
            compare["ours_vs_cub"] = round(cub_ms / ms, 3)
        except Exception as e:  # comparison only
            compare["cub_error"] = str(e)[:200]
        other = "rts" if args.algo == "csdl" else "csdl"
        with Plan(other, "u32", max_n=n) as p2:
            for _ in range(3):
                p2.scan(d_in, d_out, stream=stream)
            o_ms = time_loop(lambda: p2.scan(d_in, d_out, stream=stream), reps, stream)
            p2.check(stream)
        compare[f"{other}_gbs"] = round(alg_bytes / (o_ms * 1e-3) / 1e9, 2)
        if args.algo == "csdl":
            # The same chained scan with the decoupled fallback on (a
            # predecessor silent for 4 polls is re-reduced by its successor).
            with Plan("csdl", "u32", max_n=n) as p3:
                p3.set_fallback(4)
                for _ in range(3):
                    p3.scan(d_in, d_out, stream=stream)
                f_ms = time_loop(lambda: p3.scan(d_in, d_out, stream=stream), reps, stream)
                p3.check(stream)
            compare["csdl_fallback_gbs"] = round(alg_bytes / (f_ms * 1e-3) / 1e9, 2)

        # End to end through the C ABI from pinned host memory.
        h_out = torch.empty(n, dtype=torch.int32, pin_memory=True)
        plan.scan_host(h_in.data_ptr(), h_out.data_ptr(), n, stream=stream)
        if dist:
            dist.barrier()
        te = time.perf_counter()
        for _ in range(args.e2e_steps):
            plan.scan_host(h_in.data_ptr(), h_out.data_ptr(), n, stream=stream)
        e2e_s = (time.perf_counter() - te) / args.e2e_steps
        e2e_s = max_over_ranks(e2e_s, dist)
        # The copies alone, one direction at a time, over the same bytes: with
        # the chunks fully overlapped the end-to-end step approaches the
        # slower direction, serialised it approaches their sum.
        def copy_ms(fn):
            fn()
            torch.cuda.synchronize()
            tc = time.perf_counter()
            for _ in range(3):
                fn()
            torch.cuda.synchronize()
            return (time.perf_counter() - tc) / 3 * 1e3
        h2d_ms = copy_ms(lambda: d_out.copy_(h_in, non_blocking=True))
        d2h_ms = copy_ms(lambda: h_out.copy_(d_in, non_blocking=True))
        e2e_ms = e2e_s * 1e3
        e2e = {"value": round(world * alg_bytes / e2e_s / 1e9, 3), "unit": "GB/s", "h2d_bytes_per_step": n * 4,
               "d2h_bytes_per_step": n * 4, "ms_per_step": round(e2e_ms, 3),
               "h2d_only_ms": round(h2d_ms, 3), "d2h_only_ms": round(d2h_ms, 3),
               "overlap_of_copies": round(max(0.0, min(1.0, (h2d_ms + d2h_ms - e2e_ms) / min(h2d_ms, d2h_ms))), 3),
               "path": "gps_scan_host: pinned host -> device -> host, chunked and overlapped"}

        if not args.no_extras:
            extras["sweep"] = run_sweep(stream, d_in, d_out)
            extras["batched"] = run_batched(stream, compare.get("d2d_copy_gbs"))
            extras["fp32"] = run_fp32(stream)
            extras["mixed"] = run_mixed(stream, compare.get("d2d_copy_gbs"))
            extras["select"] = run_select(stream, compare.get("d2d_copy_gbs"))
            extras["struct"] = run_struct(stream, compare.get("d2d_copy_gbs"))

        if rank == 0 and world == 1:
            import oracle
            x = h_in.numpy().view(np.uint32)
            y = np.empty_like(x)
            reps_cpu, tc = 0, time.perf_counter()
            scan_u32 = oracle.lib().oracle_scan_u32
            while True:
                scan_u32(ctypes.c_void_p(x.ctypes.data), ctypes.c_void_p(y.ctypes.data), n, 0)
                reps_cpu += 1
                if time.perf_counter() - tc >= args.cpu_seconds and reps_cpu >= 2:
                    break
            cpu_s = (time.perf_counter() - tc) / reps_cpu
            cpu = {"value": round(alg_bytes / cpu_s / 1e9, 3), "unit": "GB/s", "cores": 1, "kind": "port",
                   "sample": f"{reps_cpu} serial scans of the full {n}-element input on one host core "
                             "(oracle/scan_oracle.c, restating Utility.hlsl:99-125)"}

    traffic_per_elem, traffic_src = profile_traffic_per_elem()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 5), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": workload_config(args, world), "algo": args.algo,
        "roofline": {"bound": "hbm", "achieved": round(kernel_gbs, 2) if kernel_gbs else None, "peak": peak,
                     "unit": "GB/s", "frac": round(kernel_gbs / peak, 4) if kernel_gbs else None,
                     "peak_kind": f"of {peak_kind}",
                     "traffic": int(traffic_per_elem * n) if traffic_per_elem else None,
                     "traffic_source": traffic_src},
        "gpu_launches": args.steps * launches,
        "clocks": clocks,
    }
    if compare:
        line["compare"] = compare
    if e2e:
        line["e2e"] = e2e
    if cpu:
        line["cpu_baseline"] = cpu
    line.update(extras)
    if "batched" in extras:
        line["batched_vs_looped_speedup"] = extras["batched"]["speedup_vs_looped_graph"]
    print(json.dumps(line), flush=True)
    plan.close()


def run_profile_case(args):
    import numpy as np
    import torch

    from gpuprefixsums_gb300 import Plan
    if args.profile_case == "batched":
        lengths = log_uniform_lengths(4096, 2 ** 20, seed=3)[:1024]
        offs = np.concatenate([[0], np.cumsum(lengths)]).astype(np.uint32)
        n = int(offs[-1])
        x = torch.randint(0, 256, (n,), dtype=torch.int32, device="cuda")
        d_off = torch.from_numpy(offs.view(np.int32)).cuda()
        with Plan("csdl", "u32", max_n=n) as plan:
            for _ in range(3):
                out = plan.scan_segmented(x, d_off)
            plan.check()
    elif args.profile_case == "select":
        n = 1 << 26
        x = torch.randint(-2 ** 31, 2 ** 31 - 1, (n,), dtype=torch.int32, device="cuda")
        fl = (torch.rand(n, device="cuda") < 0.3).to(torch.uint8)
        with Plan("csdl", "u32", max_n=n) as plan:
            for _ in range(3):
                out, cnt = plan.select(x, fl)
            plan.check()
        out = out[:int(cnt.item())]
    elif args.profile_case in ("f32c_batched", "u64_batched"):
        name = args.profile_case.split("_")[0]
        lengths = zipf_lengths(10_000, 1.2, 32, 2 ** 22, seed=5)
        kinds = np.random.default_rng(55).integers(0, 3, size=10_000)
        ls = lengths[kinds == (2 if name == "f32c" else 1)][:1000]
        offs = np.concatenate([[0], np.cumsum(ls)]).astype(np.uint32)
        n = int(offs[-1])
        x = torch.randn(n, device="cuda") if name == "f32c" else \
            torch.randint(-2 ** 63, 2 ** 63 - 1, (n,), dtype=torch.int64, device="cuda")
        d_off = torch.from_numpy(offs.view(np.int32)).cuda()
        with Plan("csdl", name, max_n=n) as plan:
            for _ in range(3):
                out = plan.scan_segmented(x, d_off)
            plan.check()
        out = out.float()
    elif args.profile_case == "mid":
        n = 1 << 20
        x = torch.randint(0, 256, (n,), dtype=torch.int32, device="cuda")
        with Plan("csdl", "u32", max_n=n) as plan:
            for _ in range(3):
                out = plan.scan(x)
            plan.check()
    elif args.profile_case == "struct":
        n = 1 << 24  # 256 MiB of structs
        x = torch.randint(-2 ** 31, 2 ** 31 - 1, (n, 4), dtype=torch.int32, device="cuda")
        with Plan("csdl", "u32x4", max_n=n) as plan:
            for _ in range(3):
                out = plan.scan(x, inclusive=True)
            plan.check()
        out = out[:, 0]
    else:
        n = 1 << 26
        x = torch.randn(n, device="cuda")
        with Plan("csdl", "f32c", max_n=n) as plan:
            for _ in range(3):
                out = plan.scan(x, inclusive=True)
            plan.check()
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": args.profile_case, "n": n, "launches": 3, "checksum": float(out[-1].item())}))


def main():
    args = parse_args()
    world, rank, local = dist_setup(args)
    if args.profile_case:
        sys.path.insert(0, ROOT)
        run_profile_case(args)
        return
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    sys.path.insert(0, ROOT)
    run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
