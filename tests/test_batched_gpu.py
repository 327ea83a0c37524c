"""Batched (segmented) scans and floating-point scans on the GPU, through the
C ABI, against the oracle.

Integer results are bit-exact (segmented oracle: oracle.segscan). Floating-
point results are compared with the exact prefix sums of the FP32 inputs
(oracle.scan_f32_exact: fixed-point superaccumulator, rounded once to FP64):
- compensated FP32: relative error of every nonzero prefix <= 1e-6 and the
  error relative to the sum of magnitudes so far (normwise) <= 1e-7 (rounding
  the exact prefix to FP32 alone costs up to 2^-24 = 6e-8 of either);
- plain FP32: normwise error <= 1e-5 (FP32 sums of up to 2^26 terms).
"""
import numpy as np
import pytest
import torch

import oracle
from gpuprefixsums_gb300 import Plan

pytestmark = pytest.mark.gpu

NP = {"u32": np.uint32, "u64": np.uint64}
TV = {"u32": np.int32, "u64": np.int64}


def dev(x):
    v = {np.dtype(np.uint32): np.int32, np.dtype(np.uint64): np.int64}.get(x.dtype, None)
    return torch.from_numpy(np.ascontiguousarray(x).view(v) if v else np.ascontiguousarray(x)).cuda()


def offsets_of(lengths):
    return np.concatenate([[0], np.cumsum(lengths)]).astype(np.uint64)


def config3_lengths(seed=3):
    # 4096 segments, lengths floor(log-uniform[1, 2^20]).
    rng = np.random.default_rng(seed)
    return np.floor(np.exp(rng.uniform(0.0, np.log(2.0 ** 20), size=4096))).astype(np.int64)


@pytest.mark.parametrize("dtype", ["u32", "u64"])
@pytest.mark.parametrize("inclusive", [False, True])
def test_segmented_random_lengths_bit_exact(cuda, dtype, inclusive):
    rng = np.random.default_rng(17)
    # Many short segments, empty ones, and some spanning several units.
    lengths = np.concatenate([rng.integers(0, 40, size=3000), rng.integers(0, 5000, size=300),
                              rng.integers(10_000, 300_000, size=12), [0, 0, 1, 1, 0]])
    rng.shuffle(lengths)
    offs = offsets_of(lengths)
    n = int(offs[-1])
    x = rng.integers(0, np.iinfo(NP[dtype]).max, size=n, dtype=NP[dtype], endpoint=True)
    want = oracle.segscan(x, offs, inclusive)
    d_off = torch.from_numpy(offs.astype(np.uint32).view(np.int32)).cuda()
    with Plan("csdl", dtype, max_n=n) as plan:
        got = plan.scan_segmented(dev(x), d_off, inclusive=inclusive)
        plan.check()
    assert np.array_equal(got.cpu().numpy().view(NP[dtype]), want)


@pytest.mark.parametrize("dtype", ["u32", "u64"])
def test_segmented_many_short_segments(cuda, dtype):
    # Hundreds of thousands of segments of 0..3 elements: every tile holds
    # hundreds of heads, and the offsets between two samples are searched.
    rng = np.random.default_rng(23)
    lengths = rng.integers(0, 4, size=600_000)
    offs = offsets_of(lengths)
    n = int(offs[-1])
    x = rng.integers(0, np.iinfo(NP[dtype]).max, size=n, dtype=NP[dtype], endpoint=True)
    d_off = torch.from_numpy(offs.astype(np.uint32).view(np.int32)).cuda()
    with Plan("csdl", dtype, max_n=n) as plan:
        for inclusive in (False, True):
            got = plan.scan_segmented(dev(x), d_off, inclusive=inclusive)
            plan.check()
            assert np.array_equal(got.cpu().numpy().view(NP[dtype]), oracle.segscan(x, offs, inclusive))


def test_segmented_config3_4096_segments_in_place(cuda):
    lengths = config3_lengths()
    offs = offsets_of(lengths)
    n = int(offs[-1])
    rng = np.random.default_rng(30)
    x = rng.integers(0, 256, size=n, dtype=np.uint32)
    want = oracle.segscan(x, offs, False)
    d = dev(x)
    d_off = torch.from_numpy(offs.astype(np.uint32).view(np.int32)).cuda()
    with Plan("csdl", "u32", max_n=n) as plan:
        plan.scan_segmented(d, d_off, out=d, inclusive=False)
        plan.check()
    assert np.array_equal(d.cpu().numpy().view(np.uint32), want)


def test_segmented_equals_looped_plain_scans_and_replays_from_a_graph(cuda):
    lengths = config3_lengths(seed=5)[:300]
    offs = offsets_of(lengths)
    n = int(offs[-1])
    rng = np.random.default_rng(31)
    x = rng.integers(0, 256, size=n, dtype=np.uint32)
    d_in = dev(x)
    d_off = torch.from_numpy(offs.astype(np.uint32).view(np.int32)).cuda()
    looped = torch.empty_like(d_in)
    with Plan("csdl", "u32", max_n=n) as plan:
        for s in range(len(lengths)):
            b, e = int(offs[s]), int(offs[s + 1])
            if e > b:
                plan.scan(d_in[b:e], looped[b:e], inclusive=False)
        batched = plan.scan_segmented(d_in, d_off)
        torch.cuda.synchronize()
        assert torch.equal(batched, looped)
        g = torch.cuda.CUDAGraph()
        st = torch.cuda.Stream()
        out = torch.empty_like(d_in)
        with torch.cuda.stream(st):
            with torch.cuda.graph(g, stream=st):
                plan.scan_segmented(d_in, d_off, out=out, stream=st)
        for _ in range(5):
            out.zero_()
            g.replay()
            torch.cuda.synchronize()
            assert torch.equal(out, looped)
        plan.check()


@pytest.mark.parametrize("max_n", [3 * 4096, 5 * 4096 + 1, 1 << 20])
def test_segmented_and_plain_scans_share_a_u32_plan(cuda, max_n):
    # Plans whose tile count is odd or even; plain scans (8-byte descriptors)
    # and batched scans (16-byte descriptors) alternate on the same plan.
    rng = np.random.default_rng(max_n)
    lengths = rng.integers(0, 3000, size=max_n // 1500)
    lengths[-1] += max_n - lengths.sum() if lengths.sum() < max_n else 0
    lengths = lengths[np.cumsum(lengths) <= max_n]
    offs = offsets_of(lengths)
    n = int(offs[-1])
    x = rng.integers(0, 2 ** 32, size=n, dtype=np.uint64).astype(np.uint32)
    d_off = torch.from_numpy(offs.astype(np.uint32).view(np.int32)).cuda()
    want_seg = oracle.segscan(x, offs, False)
    want = oracle.scan(x, inclusive=True)
    with Plan("csdl", "u32", max_n=max_n) as plan:
        for _ in range(3):
            seg = plan.scan_segmented(dev(x), d_off)
            full = plan.scan(dev(x), inclusive=True)
            plan.check()
            assert np.array_equal(seg.cpu().numpy().view(np.uint32), want_seg)
            assert np.array_equal(full.cpu().numpy().view(np.uint32), want)


@pytest.mark.parametrize("split", [1, 2])
@pytest.mark.parametrize("unit,ctas_div", [(1, 1), (4, 1), (1, 2), (4, 2)])
def test_every_launch_configuration_is_exact(cuda, unit, ctas_div, split):
    lengths = config3_lengths(seed=11)[:600]
    offs = offsets_of(lengths)
    n = int(offs[-1])
    rng = np.random.default_rng(unit * 10 + ctas_div)
    x = rng.integers(0, 2 ** 32, size=n, dtype=np.uint64).astype(np.uint32)
    d_off = torch.from_numpy(offs.astype(np.uint32).view(np.int32)).cuda()
    xf = fp_input("normal", n, seed=5)
    with Plan("csdl", "u32", max_n=n) as plan, Plan("csdl", "f32c", max_n=n) as fplan:
        plan.set_generic_config(n, unit, ctas_div, threads_per_row=split)
        fplan.set_generic_config(n, unit, ctas_div, segmented=False, threads_per_row=split)
        assert plan.generic_config(n) == {"unit_tiles": unit, "ctas_div": ctas_div, "threads_per_row": split,
                                          "tuned": True}
        for inclusive in (False, True):
            got = plan.scan_segmented(dev(x), d_off, inclusive=inclusive)
            plan.check()
            assert np.array_equal(got.cpu().numpy().view(np.uint32), oracle.segscan(x, offs, inclusive))
        got = fplan.scan(torch.from_numpy(xf).cuda(), inclusive=True).cpu().numpy()
        fplan.check()
        assert fp_errors(got, oracle.scan_f32_exact(xf, inclusive=True), xf)[0] <= 1e-6


def test_autotune_keeps_a_configuration_per_size_class(cuda):
    lengths = config3_lengths(seed=12)[:1000]
    offs = offsets_of(lengths)
    n = int(offs[-1])
    rng = np.random.default_rng(12)
    x = rng.integers(0, 256, size=n, dtype=np.uint32)
    d_off = torch.from_numpy(offs.astype(np.uint32).view(np.int32)).cuda()
    with Plan("csdl", "u32", max_n=n) as plan:
        assert not plan.generic_config(n)["tuned"]
        choice = plan.autotune(dev(x), d_off)
        cfg = plan.generic_config(n)
        assert cfg["tuned"] and {k: cfg[k] for k in choice} == choice
        assert not plan.generic_config(n // 16)["tuned"]  # another size class
        got = plan.scan_segmented(dev(x), d_off)
        plan.check()
    assert np.array_equal(got.cpu().numpy().view(np.uint32), oracle.segscan(x, offs, False))


@pytest.mark.parametrize("unit", [1, 4])
def test_generic_descriptor_layout_boundaries(cuda, unit):
    # The generic kernel gives each unit descriptor a 128-byte line for
    # launches of up to 1024 units and packs them beyond: unit counts on both
    # sides of the limit, batched u32 (exact) on one plan.
    rng = np.random.default_rng(61 + unit)
    tile = 4096
    with Plan("csdl", "u32", max_n=1100 * unit * tile) as plan:
        for units in (1024, 1025, 1023, 129, 1100):
            n = units * unit * tile - int(rng.integers(0, 100))
            lengths = rng.integers(1, 3 * tile * unit, size=max(1, n // (tile * unit)))
            lengths = np.append(lengths, 0)
            offs = np.minimum(np.concatenate([[0], np.cumsum(lengths)]), n)
            offs[-1] = n
            x = rng.integers(0, 2 ** 32, size=n, dtype=np.uint64).astype(np.uint32)
            d_off = torch.from_numpy(offs.astype(np.uint32).view(np.int32)).cuda()
            plan.set_generic_config(n, unit, 1)
            got = plan.scan_segmented(dev(x), d_off, inclusive=True)
            plan.check()
            assert np.array_equal(got.cpu().numpy().view(np.uint32), oracle.segscan(x, offs.astype(np.uint64), True)), units


# ------------------------------------------------------------ floating point
def fp_errors(got, exact, x):
    got = got.astype(np.float64)
    nz = exact != 0
    rel = np.abs(got[nz] - exact[nz]) / np.abs(exact[nz])
    if rel.size == 0:  # every exact prefix is zero (e.g. an exclusive scan of one element)
        rel = np.abs(got)
    mag = np.cumsum(np.abs(x.astype(np.float64)))
    norm = np.abs(got - exact) / np.maximum(mag, np.finfo(np.float64).tiny)
    return float(rel.max()), float(np.median(rel)), float(norm.max())


def fp_input(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "normal":
        return rng.standard_normal(n).astype(np.float32)
    mag = np.exp(rng.uniform(np.log(1e-8), np.log(1e8), size=n))
    return (mag * rng.choice([-1.0, 1.0], size=n)).astype(np.float32)


@pytest.mark.slow
@pytest.mark.parametrize("kind", ["normal", "mixed"])
def test_config4_fp32_2pow26_plain_and_compensated(cuda, kind):
    n = 1 << 26
    x = fp_input(kind, n, seed=26 if kind == "normal" else 27)
    exact = oracle.scan_f32_exact(x, inclusive=True)
    d = torch.from_numpy(x).cuda()
    res = {}
    for dt in ("f32", "f32c"):
        with Plan("csdl", dt, max_n=n) as plan:
            res[dt] = fp_errors(plan.scan(d, inclusive=True).cpu().numpy(), exact, x)
            plan.check()
    rel_c, med_c, norm_c = res["f32c"]
    print(kind, res)
    assert rel_c <= 1e-6 and norm_c <= 1e-7, res
    assert res["f32"][2] <= 1e-5, res
    assert res["f32"][0] > rel_c, res


@pytest.mark.parametrize("dt", ["f32", "f32c"])
@pytest.mark.parametrize("inclusive", [False, True])
def test_fp32_sizes_and_segments(cuda, dt, inclusive):
    rng = np.random.default_rng(4)
    for n in (1, 5, 4096, 4097, 16384 * 3 + 11, 1_000_003):
        x = fp_input("normal", n, seed=n)
        exact = oracle.scan_f32_exact(x, inclusive=inclusive)
        with Plan("csdl", dt, max_n=n) as plan:
            got = plan.scan(torch.from_numpy(x).cuda(), inclusive=inclusive).cpu().numpy()
            plan.check()
        rel, _, norm = fp_errors(got, exact, x)
        if dt == "f32c":
            assert rel <= 1e-6, (n, rel)
        else:
            assert norm <= 1e-5, (n, norm)
    # segmented, compared segment by segment with the exact prefix sums
    lengths = np.concatenate([rng.integers(0, 50, size=500), rng.integers(1000, 70_000, size=10)])
    rng.shuffle(lengths)
    offs = offsets_of(lengths)
    n = int(offs[-1])
    x = fp_input("mixed", n, seed=99)
    d_off = torch.from_numpy(offs.astype(np.uint32).view(np.int32)).cuda()
    with Plan("csdl", dt, max_n=n) as plan:
        got = plan.scan_segmented(torch.from_numpy(x).cuda(), d_off, inclusive=inclusive).cpu().numpy()
        plan.check()
    worst = 0.0
    for s in range(len(lengths)):
        b, e = int(offs[s]), int(offs[s + 1])
        if e > b:
            ex = oracle.scan_f32_exact(x[b:e], inclusive=inclusive)
            worst = max(worst, fp_errors(got[b:e], ex, x[b:e])[2])
    assert worst <= (1e-7 if dt == "f32c" else 1e-5), worst


# ------------------------------------------------------ mixed batch (config 5)
def zipf_lengths(count, s, lo, hi, seed):
    """Continuous Zipf(s) truncated to [lo, hi], floored (inverse CDF)."""
    rng = np.random.default_rng(seed)
    u = rng.uniform(0.0, 1.0, size=count)
    a, b = lo ** (1.0 - s), hi ** (1.0 - s)
    return np.clip(np.floor((a - u * (a - b)) ** (1.0 / (1.0 - s))), lo, hi).astype(np.int64)


@pytest.mark.parametrize("inclusive", [False, True])
def test_config5_mixed_batch_in_one_graph_against_the_oracle(cuda, inclusive):
    # Config 5 at reduced size: 500 scans with Zipf(1.2) lengths in
    # [32, 2^22], dtype per scan from {u32, u64, compensated f32}, batched per
    # dtype, plus a 2^22-element u32 Bernoulli(0.3) flag scan; the four
    # launches are captured in one CUDA graph and replayed twice.
    count = 500
    lengths = zipf_lengths(count, 1.2, 32, 2 ** 22, seed=50)
    kinds = np.random.default_rng(51).integers(0, 3, size=count)
    rng = np.random.default_rng(52)
    groups = {}
    for k, name in enumerate(("u32", "u64", "f32c")):
        offs = offsets_of(lengths[kinds == k])
        m = int(offs[-1])
        if name == "u32":
            x = rng.integers(0, 256, size=m, dtype=np.uint32)
        elif name == "u64":
            x = rng.integers(0, np.iinfo(np.uint64).max, size=m, dtype=np.uint64, endpoint=True)
        else:
            x = rng.standard_normal(m).astype(np.float32)
        d_x = dev(x)
        groups[name] = {"x": x, "offs": offs, "d_x": d_x, "out": torch.empty_like(d_x),
                        "d_off": torch.from_numpy(offs.astype(np.uint32).view(np.int32)).cuda(),
                        "plan": Plan("csdl", name, max_n=m)}
    nf = 1 << 22
    flags = (rng.random(nf) < 0.3).astype(np.uint32)
    d_flags, fout = dev(flags), torch.empty(nf, dtype=torch.int32, device="cuda")
    fplan = Plan("csdl", "u32", max_n=nf)
    st = torch.cuda.Stream()
    try:
        for g in groups.values():
            g["plan"].autotune(g["d_x"], g["d_off"], out=g["out"], inclusive=inclusive, stream=st)

        def batch():
            for g in groups.values():
                g["plan"].scan_segmented(g["d_x"], g["d_off"], out=g["out"], inclusive=inclusive, stream=st)
            fplan.scan(d_flags, fout, inclusive=inclusive, stream=st)

        graph = torch.cuda.CUDAGraph()
        with torch.cuda.stream(st):
            batch()
            st.synchronize()
            with torch.cuda.graph(graph, stream=st):
                batch()
        for _ in range(2):
            for g in groups.values():
                g["out"].fill_(-1)
            fout.fill_(-1)
            torch.cuda.synchronize()
            with torch.cuda.stream(st):
                graph.replay()
            st.synchronize()
            for name in ("u32", "u64"):
                g = groups[name]
                got = g["out"].cpu().numpy().view(NP[name])
                assert np.array_equal(got, oracle.segscan(g["x"], g["offs"], inclusive)), name
            assert np.array_equal(fout.cpu().numpy().view(np.uint32), oracle.scan(flags, inclusive))
            g = groups["f32c"]
            got = g["out"].cpu().numpy()
            worst_rel = worst_norm = 0.0
            for s in range(len(g["offs"]) - 1):
                b, e = int(g["offs"][s]), int(g["offs"][s + 1])
                rel, _, norm = fp_errors(got[b:e], oracle.scan_f32_exact(g["x"][b:e], inclusive=inclusive),
                                         g["x"][b:e])
                worst_rel, worst_norm = max(worst_rel, rel), max(worst_norm, norm)
            assert worst_rel <= 1e-6 and worst_norm <= 1e-7, (worst_rel, worst_norm)
        for g in groups.values():
            g["plan"].check(st)
        fplan.check(st)
    finally:
        for g in groups.values():
            g["plan"].close()
        fplan.close()
