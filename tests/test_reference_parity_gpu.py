"""Bit-exact parity with the reference's own chained-scan kernel, on the GPU.

The reference's CSDLExclusive / CSDLInclusive<8, 4>
(GPUPrefixSumsCUDA/ChainedScanDecoupledLookback.cuh:141-153), compiled from
its unmodified sources into oracle/_ref/ (oracle/build.py), is launched the
way its dispatcher does (two clearing memsets, one launch, in place:
ChainedScanDecoupledLookbackDispatcher.cuh:172-195) next to each kernel path
of this library on the same inputs:

- every n in [4096, 8192] -- the reference's own sweep
  (ChainedScanDecoupledLookbackDispatcher.cuh:48-59) -- on all-ones input and
  on the hybrid-Tausworthe input of its random tests (values & 1023, seeded
  with the size: GPUPrefixSumsD3D12/Shaders/Utility.hlsl:37-66,
  GPUPrefixSumsD3D12/GPUPrefixSumBase.h:141-147);
- seeded sizes that are not tile multiples, up to 2^20, on the same
  generator, with aligned and element-offset buffers;
- all-ones at 2^26, 2^27 and 2^28 (GPUPrefixSumBase.h:150-153);
- uniform [0, 255] up to the largest n at which every inclusive tile prefix
  the reference publishes stays below 2^30 (its descriptor keeps 30 bits,
  ChainedScanDecoupledLookback.cuh:117-119; beyond that the reference is
  wrong, see test_reference_csdl_30_bit_descriptor_limit).

Exclusive and inclusive throughout. The reference's results are checked
against the oracle as well, which pins the oracle to the reference's kernel.
"""
import numpy as np
import pytest
import torch

import oracle
from gpuprefixsums_gb300 import Plan

pytestmark = pytest.mark.gpu

PART = 4096          # the reference's tile (ChainedScanDecoupledLookbackDispatcher.cuh:13-18)
ONE_CTA_MAX = 16384  # most u32 elements the one-CTA kernel takes (64 KB)


def _ref():
    import ref_kernels
    if not ref_kernels.available():
        pytest.skip("reference kernels were not built here (no reference checkout where build() ran)")
    return ref_kernels.RefKernels()


def _paths(n):
    return (["one_cta"] if n <= ONE_CTA_MAX else []) + ["mid", "persistent"]


def _plan(path, max_n, algo="csdl"):
    plan = Plan(algo, "u32", max_n=max_n)
    plan.set_small_max(ONE_CTA_MAX if path == "one_cta" else 0)
    if path == "mid":
        plan.set_mid_max(max_n)   # one tile per CTA at every size
    if path == "persistent":
        plan.set_mid_max(0)
    return plan


def _dev(x):
    return torch.from_numpy(np.ascontiguousarray(x).view(np.int32)).cuda()


@pytest.mark.parametrize("inputs", ["ones", "tausworthe"])
@pytest.mark.parametrize("inclusive", [False, True])
def test_every_size_of_the_reference_sweep(cuda, inputs, inclusive):
    ref = _ref()
    lo, hi = PART, 2 * PART
    sizes = list(range(lo, hi + 1))
    paths = _paths(hi)
    plans = {p: _plan(p, hi) for p in paths}
    ref_buf = torch.zeros(hi + 4, dtype=torch.int32, device="cuda")
    ours = torch.zeros(hi + 4, dtype=torch.int32, device="cuda")
    tbr = torch.zeros(3, dtype=torch.int32, device="cuda")
    bump = torch.zeros(1, dtype=torch.int32, device="cuda")
    offs = np.concatenate([[0], np.cumsum(sizes)])
    ref_all = torch.empty(int(offs[-1]), dtype=torch.int32, device="cuda")
    mism = torch.zeros((len(sizes), len(paths)), dtype=torch.bool, device="cuda")
    xs = []
    try:
        for k, n in enumerate(sizes):
            x = oracle.init_one(n) if inputs == "ones" else oracle.init_random_taus(n, seed=n)
            xs.append(x)
            d_x = _dev(x)
            ref_buf[:n] = d_x
            ref.csdl_device(ref_buf, n, inclusive, tbr, bump)
            ref_all[offs[k]:offs[k] + n] = ref_buf[:n]
            for j, p in enumerate(paths):
                ours[:n] = d_x
                plans[p].scan(ours, ours, inclusive=inclusive, n=n)  # in place, as the reference
                mism[k, j] = (ours[:n] != ref_buf[:n]).any()
        for p in plans.values():
            p.check()
    finally:
        for p in plans.values():
            p.close()
    bad = mism.nonzero().tolist()
    assert not bad, [(sizes[k], paths[j]) for k, j in bad[:20]]
    # The reference kernel itself agrees with the oracle on every size.
    host = ref_all.cpu().numpy().view(np.uint32)
    wrong = [n for k, n in enumerate(sizes)
             if oracle.validate(xs[k], host[offs[k]:offs[k] + n], inclusive) != 0]
    assert not wrong, wrong[:20]


def _random_sizes():
    rng = np.random.default_rng(20)
    sizes = {8193, 12289, 16383, 16385, 65535, 65537, 528383, (1 << 20) - 1, (1 << 20) - 4095}
    while len(sizes) < 40:
        v = int(rng.integers(2 * PART + 1, 1 << 20))
        if v % PART:
            sizes.add(v)
    return sorted(sizes)


@pytest.mark.parametrize("inclusive", [False, True])
@pytest.mark.parametrize("offset", [0, 1])
def test_seeded_sizes_that_are_not_tile_multiples(cuda, inclusive, offset):
    # offset 1: input and output one element past a 16-byte boundary, so the
    # element-wise (ring / unaligned) kernels run.
    ref = _ref()
    sizes = _random_sizes()
    top = max(sizes)
    ref_buf = torch.zeros(top + 4, dtype=torch.int32, device="cuda")
    tbr = torch.zeros((top + 3) // PART + 1, dtype=torch.int32, device="cuda")
    bump = torch.zeros(1, dtype=torch.int32, device="cuda")
    buf = torch.zeros(top + 8, dtype=torch.int32, device="cuda")
    out = torch.zeros(top + 8, dtype=torch.int32, device="cuda")
    failures = []
    plans = {p: _plan(p, top) for p in ("one_cta", "mid", "persistent")}
    plans["rts"] = Plan("rts", "u32", max_n=top)
    try:
        for n in sizes:
            x = oracle.init_random_taus(n, seed=n)
            d_x = _dev(x)
            ref_buf[:n] = d_x
            ref.csdl_device(ref_buf, n, inclusive, tbr, bump)
            want = ref_buf[:n]
            assert oracle.validate(x, want.cpu().numpy().view(np.uint32), inclusive) == 0, n
            d_in = buf[offset:offset + n]
            d_in.copy_(d_x)
            d_out = out[offset:offset + n]
            for name, plan in plans.items():
                if name == "one_cta" and n > ONE_CTA_MAX:
                    continue
                d_out.fill_(-1)
                plan.scan(d_in, d_out, inclusive=inclusive)
                if not torch.equal(d_out, want):
                    failures.append((n, name))
        for p in plans.values():
            p.check()
    finally:
        for p in plans.values():
            p.close()
    assert not failures, failures[:20]


@pytest.mark.slow
@pytest.mark.parametrize("inclusive", [False, True])
def test_all_ones_at_2pow26_to_2pow28(cuda, inclusive):
    # The reference's large known-answer sizes; all-ones sums stay below
    # 2^30 up to 2^28, so its 30-bit descriptor is exact here.
    ref = _ref()
    top = 1 << 28
    ref_buf = torch.empty(top, dtype=torch.int32, device="cuda")
    ours = torch.empty(top, dtype=torch.int32, device="cuda")
    ones = torch.ones(top, dtype=torch.int32, device="cuda")
    tbr = torch.zeros(top // PART, dtype=torch.int32, device="cuda")
    bump = torch.zeros(1, dtype=torch.int32, device="cuda")
    failures = []
    plans = {p: _plan(p, top) for p in ("mid", "persistent")}
    plans["rts"] = Plan("rts", "u32", max_n=top)
    try:
        for k in (26, 27, 28):
            n = 1 << k
            ref_buf[:n].fill_(1)
            ref.csdl_device(ref_buf, n, inclusive, tbr, bump)
            want = torch.arange(int(inclusive), n + int(inclusive), dtype=torch.int32, device="cuda")
            assert torch.equal(ref_buf[:n], want), f"reference kernel at 2^{k}"  # UtilityKernels.cuh:22-38
            for name, plan in plans.items():
                ours[:n].fill_(0)
                plan.scan(ones[:n], ours[:n], inclusive=inclusive)
                if not torch.equal(ours[:n], ref_buf[:n]):
                    failures.append((k, name))
        for p in plans.values():
            p.check()
    finally:
        for p in plans.values():
            p.close()
    assert not failures, failures


def _uniform255_exact_limit(x):
    """Largest n at which every inclusive tile prefix the reference's kernel
    may read (tiles 0 .. T-2 of the T tiles of n) is below 2^30."""
    tiles = x.size // PART
    incl = np.cumsum(x[:tiles * PART].astype(np.uint64).reshape(tiles, PART).sum(axis=1))
    ok = np.nonzero(incl < (1 << 30))[0]
    last = int(ok[-1])             # last tile whose inclusive prefix fits
    return min(x.size, (last + 2) * PART)


@pytest.mark.slow
@pytest.mark.parametrize("inclusive", [False, True])
def test_uniform_0_255_up_to_the_30_bit_limit(cuda, inclusive):
    ref = _ref()
    rng = np.random.default_rng(255)
    x_all = rng.integers(0, 256, size=(1 << 23) + (1 << 21), dtype=np.uint32)
    n_max = _uniform255_exact_limit(x_all)
    assert (1 << 23) <= n_max < x_all.size
    sizes = [(1 << 22) - 1, (1 << 22) + 5, (1 << 23) - 1, n_max - PART - 1, n_max - 1, n_max]
    d_all = _dev(x_all[:n_max])
    ref_buf = torch.zeros(n_max + 4, dtype=torch.int32, device="cuda")
    tbr = torch.zeros(n_max // PART + 2, dtype=torch.int32, device="cuda")
    bump = torch.zeros(1, dtype=torch.int32, device="cuda")
    out = torch.empty(n_max, dtype=torch.int32, device="cuda")
    failures = []
    plans = {p: _plan(p, n_max) for p in ("mid", "persistent")}
    plans["rts"] = Plan("rts", "u32", max_n=n_max)
    try:
        for n in sizes:
            ref_buf[:n] = d_all[:n]
            ref.csdl_device(ref_buf, n, inclusive, tbr, bump)
            want = ref_buf[:n]
            if n == n_max:
                got_ref = want.cpu().numpy().view(np.uint32)
                assert oracle.validate(x_all[:n], got_ref, inclusive) == 0, "reference kernel at its limit"
            for name, plan in plans.items():
                plan.scan(d_all[:n], out[:n], inclusive=inclusive)
                if not torch.equal(out[:n], want):
                    failures.append((n, name))
        for p in plans.values():
            p.check()
    finally:
        for p in plans.values():
            p.close()
    assert not failures, failures
