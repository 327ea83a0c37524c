"""Stream compaction (gps_select_flagged) on the GPU against the oracle:
bit-exact outputs and counts, nothing written past the count."""
import numpy as np
import pytest
import torch

import oracle
from gpuprefixsums_gb300 import Plan

pytestmark = pytest.mark.gpu

NP = {"u32": np.uint32, "u64": np.uint64, "f32": np.uint32}
TV = {np.dtype(np.uint32): torch.int32, np.dtype(np.uint64): torch.int64}


def dev(x):
    return torch.from_numpy(x.view({4: np.int32, 8: np.int64}[x.itemsize])).cuda()


def flags_of(kind, n, rng):
    if kind == "none":
        return np.zeros(n, np.uint8)
    if kind == "all":
        return np.full(n, 7, np.uint8)
    if kind == "bernoulli":
        return (rng.random(n) < 0.3).astype(np.uint8)
    return rng.integers(0, 4, size=n, dtype=np.uint8)  # any non-zero byte selects


@pytest.mark.parametrize("dtype", ["u32", "u64", "f32"])
@pytest.mark.parametrize("kind", ["bernoulli", "bytes", "none", "all"])
def test_select_sizes_and_densities(cuda, dtype, kind):
    rng = np.random.default_rng(hash((dtype, kind)) % 2 ** 32)
    for n in (1, 15, 16, 17, 4095, 4096, 4097, 3 * 16384 + 5, 1_000_003):
        x = rng.integers(0, np.iinfo(NP[dtype]).max, size=n, dtype=NP[dtype], endpoint=True)
        fl = flags_of(kind, n, rng)
        want = oracle.select(x, fl)
        out = torch.full((n + 64,), -1, dtype=TV[np.dtype(NP[dtype])], device="cuda")  # canary past n
        with Plan("csdl", dtype, max_n=n) as plan:
            _, cnt = plan.select(dev(x), torch.from_numpy(fl).cuda(), out=out)
            plan.check()
        c = int(cnt.item())
        got = out.cpu().numpy().view(NP[dtype])
        assert c == want.size, (n, c, want.size)
        assert np.array_equal(got[:c], want), n
        assert np.all(got[c:].view({4: np.int32, 8: np.int64}[got.itemsize]) == -1), n


def test_consecutive_selects_and_scans_share_a_plan(cuda):
    # The workspace (counters, epoch, descriptors) carries over between
    # launches of the select, batched and plain kernels on one plan.
    rng = np.random.default_rng(77)
    n = 300_001
    x = rng.integers(0, 2 ** 32, size=n, dtype=np.uint64).astype(np.uint32)
    offs = np.array([0, 1000, 70_000, n], dtype=np.uint64)
    d_off = torch.from_numpy(offs.astype(np.uint32).view(np.int32)).cuda()
    with Plan("csdl", "u32", max_n=n) as plan:
        for rep in range(4):
            fl = (rng.random(n) < 0.1 * (rep + 1)).astype(np.uint8)
            out, cnt = plan.select(dev(x), torch.from_numpy(fl).cuda())
            seg = plan.scan_segmented(dev(x), d_off)
            full = plan.scan(dev(x), inclusive=True)
            plan.check()
            want = oracle.select(x, fl)
            assert int(cnt.item()) == want.size
            assert np.array_equal(out.cpu().numpy().view(np.uint32)[:want.size], want)
            assert np.array_equal(seg.cpu().numpy().view(np.uint32), oracle.segscan(x, offs, False))
            assert np.array_equal(full.cpu().numpy().view(np.uint32), oracle.scan(x, inclusive=True))


def test_select_zero_elements_writes_a_zero_count(cuda):
    cnt = torch.full((1,), 99, dtype=torch.int64, device="cuda")
    x = torch.zeros(16, dtype=torch.int32, device="cuda")
    with Plan("csdl", "u32", max_n=16) as plan:
        plan.select(x[:0], torch.zeros(0, dtype=torch.uint8, device="cuda"), num_selected=cnt)
        plan.check()
    assert int(cnt.item()) == 0


def test_select_2pow28_bernoulli_flags_and_graph_replay(cuda):
    # The flag workload of the mixed batch: 2^28 u32 values, Bernoulli(0.3)
    # flags. Checked against torch.masked_select on the device.
    n = 1 << 28
    gen = torch.Generator(device="cuda").manual_seed(28)
    x = torch.randint(-2 ** 31, 2 ** 31 - 1, (n,), dtype=torch.int32, device="cuda", generator=gen)
    fl = (torch.rand(n, device="cuda", generator=gen) < 0.3).to(torch.uint8)
    want = torch.masked_select(x, fl.bool())
    out = torch.empty_like(x)
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    with Plan("csdl", "u32", max_n=n) as plan:
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            plan.select(x, fl, out=out, num_selected=cnt, stream=s)
            s.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=s):
                plan.select(x, fl, out=out, num_selected=cnt, stream=s)
        for _ in range(3):
            with torch.cuda.stream(s):  # clear and replay on the same stream
                out.zero_()
                cnt.zero_()
                g.replay()
            s.synchronize()
            c = int(cnt.item())
            assert c == want.numel()
            assert torch.equal(out[:c], want)
        plan.check()


def test_select_argument_errors(cuda):
    from gpuprefixsums_gb300._lib import GpsError
    x = torch.zeros(1000, dtype=torch.int32, device="cuda")
    fl = torch.ones(1000, dtype=torch.uint8, device="cuda")
    with Plan("csdl", "u32", max_n=1000) as plan:
        with pytest.raises(GpsError):
            plan.select(x, fl, out=x)  # output overlaps the input
        with pytest.raises(GpsError):
            plan.select(torch.zeros(2000, dtype=torch.int32, device="cuda"),
                        torch.ones(2000, dtype=torch.uint8, device="cuda"))  # beyond max_n
    with Plan("rts", "u32", max_n=1000) as plan:
        with pytest.raises(GpsError):
            plan.select(x, fl)
