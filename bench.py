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
  cpu_baseline the oracle's serial scan on one host core.
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
PROFILE_TRAFFIC = os.path.join(ROOT, "profiles", "csdl_u32_exclusive_2pow26_ncu_full.txt")
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
    p.add_argument("--e2e-steps", type=int, default=8)
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    return p.parse_args()


# ----------------------------------------------------------------- helpers
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
    """nvidia-smi clocks and throttle reasons, sampled every 100 ms."""
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
                                          "-lms", "100", "-i", ident], stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self, t0, t1):
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
        window = [r for r in rows if t0 - 0.05 <= r[0] <= t1 + 0.05] or rows
        if not window:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "note": "no samples"}
        reasons = sorted({self.REASONS[i] for r in window for i, v in enumerate(r[3]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[1] for r in window), "sm_max_mhz": max(r[2] for r in window),
                "reasons": reasons, "samples": len(window)}


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
    rng = np.random.default_rng(2028)
    full = rng.integers(0, 256, size=args.n, dtype=np.uint32)
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
        "config": {"workload": "u32 exclusive scan of 2^28 elements, uniform [0,255], seeded",
                   "n": args.n, "sample_elements_per_step": sample},
        "cpu_baseline": {"value": round(gbs, 3), "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} of the {args.n} elements per step (3-phase reduce-then-scan "
                                   f"restated in oracle/scan_oracle.c, {threads} threads)"},
        "e2e": {"value": round(gbs, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


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
    gen = torch.Generator(device="cuda").manual_seed(2028 + rank)
    with torch.cuda.stream(stream):
        d_in = torch.randint(0, 256, (n,), dtype=torch.int32, device="cuda", generator=gen)
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
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.time()
    ms = time_loop(step, args.steps, stream)
    torch.cuda.synchronize()
    t1 = time.time()
    if dist:
        dist.barrier()
    clocks = sampler.stop(t0, t1)
    plan.check(stream)
    if dist:
        t = torch.tensor([ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    alg_bytes = n * 8
    value = world * alg_bytes / (ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak()
    kernel_gbs = alg_bytes / (ms / launches * 1e-3) / 1e9 if launches == 1 else None

    compare, e2e, cpu = {}, None, None
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

        # End to end through the C ABI from pinned host memory.
        h_in = torch.empty(n, dtype=torch.int32, pin_memory=True)
        h_out = torch.empty(n, dtype=torch.int32, pin_memory=True)
        h_in.copy_(d_in.cpu())
        plan.scan_host(h_in.data_ptr(), h_out.data_ptr(), n, stream=stream)
        if dist:
            dist.barrier()
        te = time.perf_counter()
        for _ in range(args.e2e_steps):
            plan.scan_host(h_in.data_ptr(), h_out.data_ptr(), n, stream=stream)
        e2e_s = (time.perf_counter() - te) / args.e2e_steps
        if dist:
            t = torch.tensor([e2e_s], device="cuda", dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            e2e_s = float(t.item())
        e2e = {"value": round(world * alg_bytes / e2e_s / 1e9, 3), "unit": "GB/s", "h2d_bytes_per_step": n * 4,
               "d2h_bytes_per_step": n * 4, "ms_per_step": round(e2e_s * 1e3, 3),
               "path": "gps_scan_host: pinned host -> device -> host, chunked and overlapped"}

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
        "config": {"workload": f"u32 exclusive scan, n={n}, {args.algo}, out of place, uniform [0,255] seeded",
                   "n": n, "algo": args.algo, "parallelism": f"replicas x{world}",
                   "l2": "inputs and outputs of 1 GiB each exceed the 129 MB L2; no flush needed"},
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
    print(json.dumps(line), flush=True)
    plan.close()


def main():
    args = parse_args()
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    sys.path.insert(0, ROOT)
    run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
