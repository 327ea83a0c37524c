"""Parity of the CUDA scans (through the C ABI) with the oracle, on the GPU.

Bit-exact for every case: u32 and u64 scans wrap mod 2^w. Small and medium
sizes are compared element by element with the serial oracle; 2^28 is
compared in full as well (the oracle needs under a second for it).
"""
import numpy as np
import pytest
import torch

import oracle
from gpuprefixsums_gb300 import GpsError, Plan, _lib

pytestmark = pytest.mark.gpu

ALGOS = ["csdl", "rts"]
TILE = {"u32": 4096, "u64": 2048}
NP = {"u32": np.uint32, "u64": np.uint64}
TORCH_VIEW = {"u32": (np.int32, torch.int32), "u64": (np.int64, torch.int64)}


# Kernel paths of an integer scan: the one-CTA scan of small inputs, the
# one-tile-per-CTA chained scan of mid sizes, and the persistent kernels.
PATHS = ["one_cta", "mid", "persistent"]


def use_path(plan, algo, path):
    """Route every size of the test through one kernel path (the defaults
    send each size to the path its size class takes)."""
    if path == "mid" and algo != "csdl":
        pytest.skip("the mid-size kernel serves chained-scan plans")
    # The one-CTA kernel takes up to 64 KB of input; chained-scan plans
    # leave it off by default.
    plan.set_small_max(65536 // plan.elem_size if path == "one_cta" else 0)
    if path == "persistent":
        plan.set_mid_max(0)


def to_dev(x: np.ndarray) -> torch.Tensor:
    view = np.int32 if x.dtype == np.uint32 else np.int64
    return torch.from_numpy(np.ascontiguousarray(x).view(view)).cuda()


def to_host(t: torch.Tensor, dtype) -> np.ndarray:
    return t.cpu().numpy().view(dtype)


def rand(dtype, n, seed, high=None):
    rng = np.random.default_rng(seed)
    if dtype == "u32":
        hi = (1 << 32) if high is None else high
        return rng.integers(0, hi, size=n, dtype=np.uint64).astype(np.uint32)
    hi = np.iinfo(np.uint64).max if high is None else high - 1
    return rng.integers(0, hi, size=n, dtype=np.uint64, endpoint=True)


# --------------------------------------------------------------- config 1
@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("inclusive", [False, True])
def test_config1_2pow20_uniform_0_15(cuda, algo, inclusive):
    # n = 2^20 u32 drawn from U[0, 15] with a fixed seed, CSDL and RTS.
    x = rand("u32", 1 << 20, seed=20240601, high=16)
    with Plan(algo, "u32", max_n=1 << 20) as plan:
        out = plan.scan(to_dev(x), inclusive=inclusive)
        plan.check()
    assert oracle.validate(x, to_host(out, np.uint32), inclusive) == 0


# -------------------------------------------- the reference's size sweep
@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("inclusive", [False, True])
@pytest.mark.parametrize("path", PATHS)
def test_every_size_from_one_to_two_tiles_all_ones_in_place(cuda, algo, inclusive, path):
    # ChainedScanDecoupledLookbackDispatcher.cuh:48-59: every n in
    # [4096, 8192] on all-ones input, scanned in place; extended down to 1.
    # Through each kernel path.
    top = 2 * 4096 + 1
    with Plan(algo, "u32", max_n=top) as plan:
        use_path(plan, algo, path)
        buf = torch.empty(top, dtype=torch.int32, device="cuda")
        ar = torch.arange(top + 1, dtype=torch.int64, device="cuda")
        bad = []
        for n in range(1, top + 1):
            buf[:n].fill_(1)
            plan.scan(buf, buf, inclusive=inclusive, n=n)
            want = ar[1:n + 1] if inclusive else ar[:n]
            if not torch.equal(buf[:n].to(torch.int64), want):
                bad.append(n)
        plan.check()
    assert not bad, f"wrong sizes: {bad[:20]}"


@pytest.mark.parametrize("dtype", ["u32", "u64"])
@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("inclusive", [False, True])
@pytest.mark.parametrize("path", PATHS)
def test_random_sizes_full_range_with_canary(cuda, dtype, algo, inclusive, path):
    # Full-range values (sums wrap), out of place, and words after n must
    # stay untouched (the reference writes up to align4(n)).
    rng = np.random.default_rng(99)
    t = TILE[dtype]
    sizes = sorted(set([1, 2, 3, 4, 5, 7, 15, 16, 17, t - 1, t, t + 1, 2 * t + 3, 5 * t - 1] +
                       rng.integers(1, 40 * t, size=12).tolist()))
    canary = 64
    with Plan(algo, dtype, max_n=max(sizes)) as plan:
        use_path(plan, algo, path)
        for n in sizes:
            x = rand(dtype, n, seed=n)
            d_in = to_dev(x)
            out_full = torch.full((n + canary,), -0x5A5A5A5B, dtype=TORCH_VIEW[dtype][1], device="cuda")
            before = out_full[n:].clone()
            plan.scan(d_in, out_full, inclusive=inclusive, n=n)
            plan.check()
            got = to_host(out_full[:n], NP[dtype])
            assert oracle.validate(x, got, inclusive) == 0, (dtype, algo, n)
            assert torch.equal(out_full[n:], before), f"wrote past n={n}"


@pytest.mark.parametrize("dtype", ["u32", "u64"])
@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("path", PATHS)
def test_unaligned_pointers_take_the_plain_path(cuda, dtype, algo, path):
    # Pointers aligned to the element but not to 16 bytes; in and out offset
    # differently.
    es = 4 if dtype == "u32" else 8
    t = TILE[dtype]
    for n in (1, 3, t + 5, 7 * t + 1):
        x = rand(dtype, n, seed=3 * n + 1)
        big_in = torch.zeros(n + 8, dtype=TORCH_VIEW[dtype][1], device="cuda")
        big_out = torch.zeros(n + 8, dtype=TORCH_VIEW[dtype][1], device="cuda")
        big_in[1:n + 1] = to_dev(x)
        with Plan(algo, dtype, max_n=n) as plan:
            use_path(plan, algo, path)
            plan.scan_ptr(big_in.data_ptr() + es, big_out.data_ptr() + 3 * es, n, inclusive=False)
            plan.check()
        got = to_host(big_out[3:n + 3], NP[dtype])
        assert oracle.validate(x, got, False) == 0, n
        assert int(big_out[:3].abs().sum()) == 0 and int(big_out[n + 3:].abs().sum()) == 0


@pytest.mark.parametrize("algo", ALGOS)
def test_u64_2pow27(cuda, algo):
    # The u64 variant at n = 2^27, full-range values.
    n = 1 << 27
    x = rand("u64", n, seed=27)
    with Plan(algo, "u64", max_n=n) as plan:
        out = plan.scan(to_dev(x), inclusive=False)
        plan.check()
    assert oracle.validate(x, to_host(out, np.uint64), False) == 0


# ------------------------------------- descriptor layouts at their limits
@pytest.mark.parametrize("dtype", ["u32", "u64"])
def test_mid_descriptor_layout_boundaries(cuda, dtype):
    # The one-tile-per-CTA kernel packs tile descriptors 8 to a 128-byte line
    # for launches of up to 32 tiles and gives each its own line from 33 to
    # 4096 tiles; past 4096 (mid_max raised) they are packed again. Launches
    # of each layout in a row on one plan, tile counts on both sides of each
    # limit, ragged last tiles.
    t = TILE[dtype]
    tiles = [32, 33, 4096, 4097, 1, 2, 31, 64, 4095]
    top = max(tiles) * t
    with Plan("csdl", dtype, max_n=top) as plan:
        plan.set_small_max(0)
        plan.set_mid_max(top)
        for k, nt in enumerate(tiles):
            n = nt * t - (k % 3) * 7
            x = rand(dtype, n, seed=500 + k)
            out = plan.scan(to_dev(x), inclusive=bool(k & 1))
            plan.check()
            assert oracle.validate(x, to_host(out, NP[dtype]), bool(k & 1)) == 0, (dtype, nt)


# ---------------------------------------------------------- config 2 sweep
def _config2_sizes():
    rng = np.random.default_rng(2)
    sizes = set()
    for k in range(10, 29):
        sizes.update({(1 << k) - 1, 1 << k, (1 << k) + 1})
    for d in range(3, 9):
        lo, hi = 10 ** d, min(10 ** (d + 1), 1 << 28)
        while True:
            v = int(rng.integers(lo, hi))
            if v % 4096:
                sizes.add(v)
                break
    return sorted(s for s in sizes if s <= (1 << 28) + 1)


@pytest.mark.slow
@pytest.mark.parametrize("dist", ["uniform255", "ones", "fullrange"])
def test_config2_exclusive_sweep_2pow10_to_2pow28(cuda, dist):
    sizes = _config2_sizes()
    top = max(sizes)
    rng_seed = {"uniform255": 255, "ones": 1, "fullrange": 32}[dist]
    if dist == "ones":
        x_all = np.ones(top, dtype=np.uint32)
    elif dist == "uniform255":
        x_all = rand("u32", top, seed=rng_seed, high=256)
    else:
        x_all = rand("u32", top, seed=rng_seed)
    d_all = to_dev(x_all)
    out = torch.empty(top, dtype=torch.int32, device="cuda")
    ref_all = oracle.scan(x_all, inclusive=False)
    with Plan("csdl", "u32", max_n=top) as plan:
        for n in sizes:
            plan.scan(d_all, out, inclusive=False, n=n)
            plan.check()
            got = to_host(out[:n], np.uint32)
            # The exclusive scan of a prefix of x is the prefix of the scan.
            assert np.array_equal(got, ref_all[:n]), (dist, n)


# ------------------------------------------------------------ host arrays
@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("inclusive", [False, True])
@pytest.mark.parametrize("path", ["mid", "persistent"])
def test_host_array_scan_chunks_and_carries(cuda, algo, inclusive, path):
    n = (1 << 24) + 12345  # the plan's 2^21 bound forces nine chunks: the six staging buffers wrap
    x = rand("u32", n, seed=5)
    h_in = torch.from_numpy(x.view(np.int32)).pin_memory()
    h_out = torch.empty(n, dtype=torch.int32).pin_memory()
    with Plan(algo, "u32", max_n=1 << 21) as plan:
        use_path(plan, algo, path)
        plan.scan_host(h_in.data_ptr(), h_out.data_ptr(), n, inclusive=inclusive)
        plan.check()
    assert oracle.validate(x, h_out.numpy().view(np.uint32), inclusive) == 0
    # in place on the host
    with Plan(algo, "u32", max_n=1 << 21) as plan:
        use_path(plan, algo, path)
        plan.scan_host(h_in.data_ptr(), h_in.data_ptr(), n, inclusive=inclusive)
    assert oracle.validate(x, h_in.numpy().view(np.uint32), inclusive) == 0


# --------------------------------------- repeated launches and graph replay
def test_many_consecutive_launches_reuse_the_workspace(cuda):
    rng = np.random.default_rng(8)
    with Plan("csdl", "u32", max_n=1 << 22) as plan:
        for i in range(60):
            n = int(rng.integers(1, 1 << 22))
            x = rand("u32", n, seed=1000 + i)
            out = plan.scan(to_dev(x), inclusive=bool(i & 1))
            assert oracle.validate(x, to_host(out, np.uint32), bool(i & 1)) == 0, (i, n)
        plan.check()


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("path", ["mid", "persistent"])
def test_cuda_graph_capture_and_replay(cuda, algo, path):
    n = 3_000_001
    x = rand("u32", n, seed=77)
    d_in = to_dev(x)
    d_out = torch.empty_like(d_in)
    ref = oracle.scan(x, inclusive=True)
    with Plan(algo, "u32", max_n=n) as plan:
        use_path(plan, algo, path)
        plan.scan(d_in, d_out, inclusive=True)  # warm-up outside capture
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                plan.scan(d_in, d_out, inclusive=True, stream=s)
        for _ in range(10):
            d_out.zero_()
            g.replay()
            torch.cuda.synchronize()
            assert np.array_equal(to_host(d_out, np.uint32), ref)
        plan.check()


# ---------------------------------------------------- forced-stall runs
@pytest.mark.parametrize("dtype", ["u32", "u64"])
def test_forced_stall_reference_pattern_with_fallback(cuda, dtype):
    # EmulatedDeadlocking.cuh:64-150: every 8th tile withholds its aggregate
    # until a successor, after 4 empty polls, re-reduces it and inserts it.
    n = 300 * TILE[dtype] + 17
    x = rand(dtype, n, seed=8)
    with Plan("csdl", dtype, max_n=n) as plan:
        plan.set_stall(mode=1, period=8, seed=0, delay_ns=20_000_000, fallback_polls=4)
        out = plan.scan(to_dev(x), inclusive=True)
        plan.check()
        st = plan.stats()
    assert oracle.validate(x, to_host(out, NP[dtype]), True) == 0
    # Stalls count lookback units (a few tiles each): every 8th of them.
    assert st["stalls"] >= 300 // (8 * 4)
    assert st["fallbacks"] > 0 and st["inserts"] > 0


@pytest.mark.parametrize("dtype", ["u32", "u64"])
def test_decoupled_fallback_mode_is_exact(cuda, dtype):
    # Production fallback (no forced stalls): aggressive re-reduction after a
    # single empty poll, in and out of place, aligned and unaligned buffers.
    for n in (1, 4097, 50 * TILE[dtype] + 3, 1 << 22):
        x = rand(dtype, n, seed=n)
        want = oracle.scan(x, inclusive=False)
        with Plan("csdl", dtype, max_n=n + 4) as plan:
            plan.set_fallback(1)
            d = to_dev(x)
            out = plan.scan(d, inclusive=False)
            plan.scan(d, out=d, inclusive=False)  # in place
            plan.check()
            assert np.array_equal(to_host(out, NP[dtype]), want), n
            assert np.array_equal(to_host(d, NP[dtype]), want), n
            if n > 2:
                buf = to_dev(np.concatenate([x[:1], x]))  # element-aligned, not 16-byte aligned
                un = buf[1:]
                res = plan.scan(un, out=un, inclusive=False)
                plan.check()
                assert np.array_equal(to_host(res, NP[dtype]), want), n
            plan.set_fallback(0)


@pytest.mark.parametrize("inclusive", [False, True])
def test_forced_stall_seeded_delays_without_fallback(cuda, inclusive):
    # Seeded random tiles are delayed by 30 us; successors just wait.
    n = (1 << 22) + 3
    x = rand("u32", n, seed=9)
    with Plan("csdl", "u32", max_n=n) as plan:
        plan.set_stall(mode=2, period=16, seed=12345, delay_ns=30_000, fallback_polls=0)
        out = plan.scan(to_dev(x), inclusive=inclusive)
        plan.check()
        st = plan.stats()
    assert oracle.validate(x, to_host(out, np.uint32), inclusive) == 0
    assert st["stalls"] > 0 and st["fallbacks"] == 0


def test_expired_wait_is_reported_and_the_plan_stays_usable(cuda):
    # Tiles withhold their aggregate for 5 ms while successors may only wait
    # 50 us: the lookback gives up, flags the plan, and the kernel ends.
    n = 64 * 4096
    x = rand("u32", n, seed=10)
    with Plan("csdl", "u32", max_n=n) as plan:
        plan.set_wait_budget(50_000)
        plan.set_stall(mode=1, period=4, seed=0, delay_ns=5_000_000, fallback_polls=0)
        plan.scan(to_dev(x), inclusive=False)
        assert plan.check_status() == _lib.GPS_ERR_TIMEOUT
        # Back to normal on the same plan.
        plan.set_stall(mode=0)
        plan.set_wait_budget(1_000_000_000)
        out = plan.scan(to_dev(x), inclusive=False)
        plan.check()
    assert oracle.validate(x, to_host(out, np.uint32), False) == 0


# ------------------------------------------------------------- arguments
def test_argument_errors_mirror_the_reference(cuda):
    with Plan("csdl", "u32", max_n=1000) as plan:
        d = torch.zeros(2000, dtype=torch.int32, device="cuda")
        with pytest.raises(GpsError) as e:
            plan.scan(d, n=1001)
        assert e.value.status == _lib.GPS_ERR_SIZE_EXCEEDS_PLAN
        with pytest.raises(GpsError) as e:  # partial overlap
            plan.scan_ptr(d.data_ptr(), d.data_ptr() + 8, 100)
        assert e.value.status == _lib.GPS_ERR_INVALID_ARGUMENT
        with pytest.raises(GpsError) as e:  # not aligned to the element
            plan.scan_ptr(d.data_ptr() + 2, d.data_ptr() + 4000, 100)
        assert e.value.status == _lib.GPS_ERR_INVALID_ARGUMENT
        plan.scan(d, n=0)  # no-op
        plan.check()


# --------------------------------------- the reference's own kernels
def _ref():
    import ref_kernels
    if not ref_kernels.available():
        pytest.skip("reference kernels were not built here (no reference checkout where build() ran)")
    return ref_kernels.RefKernels()


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("inclusive", [False, True])
def test_reference_csdl_agrees_on_config1(cuda, algo, inclusive):
    # Config 1 (2^20 u32, U[0,15]): the reference's chained scan, this
    # library (both algorithms) and the oracle agree bit for bit.
    ref = _ref()
    x = rand("u32", 1 << 20, seed=20240601, high=16)
    want = ref.scan("csdl", x, inclusive)
    assert oracle.validate(x, want, inclusive) == 0  # pins the oracle
    with Plan(algo, "u32", max_n=1 << 20) as plan:
        got = to_host(plan.scan(to_dev(x), inclusive=inclusive), np.uint32)
    assert np.array_equal(got, want)


# The reference's SpineScan adds the whole block's total s_red[WARPS - 1]
# instead of the preceding warps' s_red[WARP_INDEX - 1] for warps >= 1
# (ReduceThenScan.cuh:91-92), so its reduce-then-scan is exact only while the
# spine fits in warp 0: up to 129 tiles of 4096, n <= 528384.
REF_RTS_EXACT_MAX_N = 129 * 4096


@pytest.mark.parametrize("inclusive", [False, True])
def test_reference_rts_agrees_where_its_spine_is_exact(cuda, inclusive):
    # Full-range values: the reference's reduce-then-scan keeps 32-bit tile
    # sums, so it wraps mod 2^32 exactly like the oracle and this library.
    ref = _ref()
    rng = np.random.default_rng(4)
    for n in (1, 3, 4095, 4096, 4097, 12289, 100_003, 300_000, REF_RTS_EXACT_MAX_N):
        x = rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)
        want = ref.scan("rts", x, inclusive)
        assert oracle.validate(x, want, inclusive) == 0, n
        with Plan("rts", "u32", max_n=n) as p1, Plan("csdl", "u32", max_n=n) as p2:
            assert np.array_equal(to_host(p1.scan(to_dev(x), inclusive=inclusive), np.uint32), want)
            assert np.array_equal(to_host(p2.scan(to_dev(x), inclusive=inclusive), np.uint32), want)


@pytest.mark.parametrize("inclusive", [False, True])
def test_reference_rts_spine_defect_beyond_129_tiles(cuda, inclusive):
    # Config 1 size, 256 tiles: the reference's reduce-then-scan is right on
    # tiles 0..128 and wrong from tile 129 on; this library's is right
    # everywhere.
    ref = _ref()
    x = rand("u32", 1 << 20, seed=20240601, high=16)
    want = oracle.scan(x, inclusive)
    theirs = ref.scan("rts", x, inclusive)
    with Plan("rts", "u32", max_n=x.size) as plan:
        ours = to_host(plan.scan(to_dev(x), inclusive=inclusive), np.uint32)
    assert np.array_equal(ours, want)
    assert np.array_equal(theirs[:REF_RTS_EXACT_MAX_N], want[:REF_RTS_EXACT_MAX_N])
    assert not np.array_equal(theirs[REF_RTS_EXACT_MAX_N:], want[REF_RTS_EXACT_MAX_N:])


def test_reference_csdl_30_bit_descriptor_limit(cuda):
    # The reference's chained scan packs a 30-bit payload into its tile
    # descriptor (ChainedScanDecoupledLookback.cuh:117-119): once an inclusive
    # tile prefix reaches 2^30 its output differs from the true scan by a
    # multiple of 2^30. This library keeps the full 32-bit value.
    ref = _ref()
    n = 16 * 4096
    x = np.full(n, 1 << 18, dtype=np.uint32)  # each later tile sums to 2^30
    x[:4096] = 1
    want = oracle.scan(x, inclusive=True)
    theirs = ref.scan("csdl", x, True)
    with Plan("csdl", "u32", max_n=n) as plan:
        ours = to_host(plan.scan(to_dev(x), inclusive=True), np.uint32)
    assert np.array_equal(ours, want)
    diff = (theirs.astype(np.int64) - want.astype(np.int64)) % (1 << 32)
    assert np.all(diff % (1 << 30) == 0)
    assert np.array_equal(theirs[:4096], want[:4096])  # tile 0 needs no descriptor
    assert np.any(diff != 0)


# ------------------------------------------------------ kernel selection
def test_mid_size_scans_take_one_tile_per_cta(cuda):
    # Above the one-CTA size and up to the plan's mid size, a chained scan
    # launches one CTA per 16 KB tile; past it, the persistent kernel.
    n = (1 << 20) - 7
    x = rand("u32", n, seed=41)
    with Plan("csdl", "u32", max_n=n) as plan:
        out = plan.scan(to_dev(x))
        assert plan.geometry(n)["grid"] == (n + 4095) // 4096
        assert oracle.validate(x, to_host(out, np.uint32), False) == 0
        plan.set_mid_max(1 << 16)
        out = plan.scan(to_dev(x))
        assert plan.geometry(n)["grid"] <= 2 * torch.cuda.get_device_properties(0).multi_processor_count
        assert oracle.validate(x, to_host(out, np.uint32), False) == 0
        plan.check()


def test_mid_max_takes_integer_chained_scan_plans_only(cuda):
    for algo, dtype in (("rts", "u32"), ("csdl", "f32"), ("csdl", "u32x4")):
        with Plan(algo, dtype, max_n=1024) as plan:
            plan.set_mid_max(0)
            with pytest.raises(GpsError) as e:
                plan.set_mid_max(1024)
            assert e.value.status == _lib.GPS_ERR_UNSUPPORTED


def test_mid_size_scans_beside_a_kernel_holding_half_the_sms(cuda):
    # The one-tile-per-CTA kernel takes tile ids from the block index when
    # its grid fits the GPU at once; a CTA then waits only on lower block
    # indices, which the hardware starts first. Here another stream's kernel
    # holds half of the SMs (all of their shared memory) while mid-size scans
    # run, so only part of each grid is resident at a time: the results stay
    # exact and no wait runs out.
    import ctypes

    from gpuprefixsums_gb300 import build as B
    dl = ctypes.CDLL(B.build_device_tests())
    dl.gps_devtest_occupy.argtypes = [ctypes.c_uint, ctypes.c_ulonglong, ctypes.c_void_p]
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    side, main = torch.cuda.Stream(), torch.cuda.Stream()
    sizes = [(1 << 20) - 5, 1 << 20, 600_001, 3 * 4096 * 40 + 7]
    xs = [rand("u32", n, seed=n) for n in sizes]
    d_in = [to_dev(x) for x in xs]
    outs = [torch.empty_like(d) for d in d_in]
    with Plan("csdl", "u32", max_n=1 << 20) as plan:
        plan.set_small_max(0)
        for _ in range(3):
            torch.cuda.synchronize()
            assert dl.gps_devtest_occupy(sms // 2, 30_000_000, ctypes.c_void_p(side.cuda_stream)) == 0
            for d, o, n in zip(d_in, outs, sizes):
                for inclusive in (False, True):
                    plan.scan(d, o, inclusive=inclusive, n=n, stream=main)
            main.synchronize()
            plan.check(main)
            for x, o in zip(xs, outs):
                assert oracle.validate(x, to_host(o, np.uint32), True) == 0
        side.synchronize()
