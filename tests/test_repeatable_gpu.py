"""The generic kernel's lookback sums every prefix in a fixed order:
repeated floating-point scans with the same inputs and launch configuration
are bitwise identical, and within the error bounds against the exact prefix
sums (compensated FP32: relative error <= 1e-6; plain FP32: normwise error
<= 1e-5). Integer batched scans, whose prefixes fold segment heads in that
order, are bit-exact against the oracle for every launch configuration.
"""
import numpy as np
import pytest
import torch

import oracle
from gpuprefixsums_gb300 import Plan
from test_batched_gpu import config3_lengths, dev, fp_errors, fp_input, offsets_of

pytestmark = pytest.mark.gpu

CONFIGS = [(1, 1, 1), (4, 1, 1), (1, 2, 2), (4, 1, 2)]  # (tiles per unit, CTA divisor, threads per row)


def _repeat(plan, fn, runs):
    outs = []
    for _ in range(runs):
        outs.append(fn().cpu().numpy().copy())
        plan.check()
    return outs


@pytest.mark.parametrize("dt", ["f32", "f32c"])
@pytest.mark.parametrize("cfg", CONFIGS)
def test_fp_scan_is_bitwise_repeatable(cuda, dt, cfg):
    unit, ctas_div, split = cfg
    # 3 x 2^22 + 77 elements: 3073 tiles, so 25 groups of 128 single-tile
    # units or 7 groups of four-tile units, and a ragged last tile.
    n = 3 * (1 << 22) + 77
    x = fp_input("mixed", n, seed=41)
    d = torch.from_numpy(x).cuda()
    exact = oracle.scan_f32_exact(x, inclusive=True)
    with Plan("csdl", dt, max_n=n) as plan:
        plan.set_generic_config(n, unit, ctas_div, segmented=False, threads_per_row=split)
        outs = _repeat(plan, lambda: plan.scan(d, inclusive=True), 4)
    for o in outs[1:]:
        assert np.array_equal(o.view(np.uint32), outs[0].view(np.uint32))
    rel, _, norm = fp_errors(outs[0], exact, x)
    if dt == "f32c":
        assert rel <= 1e-6, rel
    else:
        assert norm <= 1e-5, norm


@pytest.mark.parametrize("dt", ["f32", "f32c"])
@pytest.mark.parametrize("inclusive", [False, True])
def test_fp_batched_scan_is_bitwise_repeatable(cuda, dt, inclusive):
    rng = np.random.default_rng(8)
    lengths = np.concatenate([rng.integers(0, 50, size=2000), rng.integers(1000, 200_000, size=40), [0, 1]])
    rng.shuffle(lengths)
    offs = offsets_of(lengths)
    n = int(offs[-1])
    x = fp_input("mixed", n, seed=98)
    d = torch.from_numpy(x).cuda()
    d_off = torch.from_numpy(offs.astype(np.uint32).view(np.int32)).cuda()
    with Plan("csdl", dt, max_n=n) as plan:
        plan.set_generic_config(n, 1, 1)
        outs = _repeat(plan, lambda: plan.scan_segmented(d, d_off, inclusive=inclusive), 3)
    for o in outs[1:]:
        assert np.array_equal(o.view(np.uint32), outs[0].view(np.uint32))
    worst = 0.0
    for s in range(len(lengths)):
        b, e = int(offs[s]), int(offs[s + 1])
        if e > b:
            ex = oracle.scan_f32_exact(x[b:e], inclusive=inclusive)
            worst = max(worst, fp_errors(outs[0][b:e], ex, x[b:e])[2])
    assert worst <= (1e-7 if dt == "f32c" else 1e-5), worst


@pytest.mark.parametrize("dtype", ["u32", "u64"])
@pytest.mark.parametrize("cfg", CONFIGS)
def test_integer_batched_scan_is_exact(cuda, dtype, cfg):
    unit, ctas_div, split = cfg
    np_t = {"u32": np.uint32, "u64": np.uint64}[dtype]
    rng = np.random.default_rng(31 + unit)
    # Short segments (heads in most units), long ones (groups of units with no
    # head, whose prefixes come from the group chain), and empty ones.
    lengths = np.concatenate([rng.integers(0, 40, size=4000), rng.integers(0, 5000, size=300),
                              config3_lengths(seed=5)[:60], [0, 0, 1]])
    rng.shuffle(lengths)
    offs = offsets_of(lengths)
    n = int(offs[-1])
    x = rng.integers(0, np.iinfo(np_t).max, size=n, dtype=np_t, endpoint=True)
    d_off = torch.from_numpy(offs.astype(np.uint32).view(np.int32)).cuda()
    with Plan("csdl", dtype, max_n=n) as plan:
        plan.set_generic_config(n, unit, ctas_div, threads_per_row=split)
        for inclusive in (False, True):
            got = plan.scan_segmented(dev(x), d_off, inclusive=inclusive)
            plan.check()
            assert np.array_equal(got.cpu().numpy().view(np_t), oracle.segscan(x, offs, inclusive))


def test_integer_scans_of_changing_sizes_on_one_plan(cuda):
    # Group descriptors of an earlier, larger launch are still in memory when
    # a smaller one runs: the launch tag keeps them from being read.
    rng = np.random.default_rng(77)
    big = 1 << 23
    x = rng.integers(0, 2 ** 32, size=big, dtype=np.uint64).astype(np.uint32)
    with Plan("csdl", "u32x4", max_n=big // 4) as splan, Plan("csdl", "u32", max_n=big) as plan:
        for n in (big, 4096 * 129 + 5, big - 3, 70_000, big):
            offs = np.array([0, n // 3, n // 3, n], dtype=np.uint64)
            d_off = torch.from_numpy(offs.astype(np.uint32).view(np.int32)).cuda()
            got = plan.scan_segmented(dev(x[:n]), d_off, inclusive=True)
            plan.check()
            assert np.array_equal(got.cpu().numpy().view(np.uint32), oracle.segscan(x[:n], offs, True)), n
            m = n // 4
            xs = x[:4 * m].reshape(m, 4)
            got = splan.scan(dev(xs.reshape(-1)), inclusive=False, n=m)
            splan.check()
            want = oracle.scan_members(xs, inclusive=False)
            assert np.array_equal(got.cpu().numpy().view(np.uint32).reshape(m, 4), want), n
