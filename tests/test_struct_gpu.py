"""Struct scans (GPS_DTYPE_U32X4: four independent u32 members per element)
on the GPU, through the C ABI, against the oracle (oracle.scan_members) and
the reference's known answer for all-ones input
(GPUPrefixSumsWebGPUapis/SharedShaders/validate.wgsl:51-59). Bit-exact.
"""
import numpy as np
import pytest
import torch

import oracle
from gpuprefixsums_gb300 import Plan
from gpuprefixsums_gb300._lib import GPS_ERR_INVALID_ARGUMENT, GPS_ERR_UNSUPPORTED, GpsError

pytestmark = pytest.mark.gpu

STRUCT_TILE = 1024  # 16 KB tiles of 16-byte structs


def dev(x):
    return torch.from_numpy(np.ascontiguousarray(x, dtype=np.uint32).view(np.int32)).cuda()


def host(t):
    return t.cpu().numpy().view(np.uint32)


def random_structs(n, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(0, 1 << 32, size=(n, 4), dtype=np.uint64).astype(np.uint32)


@pytest.mark.parametrize("structs", [1, 5, 8, 1023, 1024, 1025, 4 * STRUCT_TILE + 7, 1 << 16, (1 << 20) + 3])
def test_all_ones_known_answer(cuda, structs):
    with Plan("csdl", "u32x4", max_n=structs) as plan:
        got = plan.scan(torch.ones(structs, 4, dtype=torch.int32, device="cuda"), inclusive=True)
        plan.check()
    assert np.array_equal(host(got).reshape(-1), oracle.expected_struct_ones(4 * structs))


SIZES = [1, 2, 7, 8, 9, 127, 128, 129, STRUCT_TILE - 1, STRUCT_TILE, STRUCT_TILE + 1, 3 * 4 * STRUCT_TILE + 5,
         (1 << 18) + 11, (1 << 21) + 1]


@pytest.mark.parametrize("structs", SIZES)
@pytest.mark.parametrize("inclusive", [False, True])
def test_random_structs_bit_exact(cuda, structs, inclusive):
    x = random_structs(structs, seed=structs)
    with Plan("csdl", "u32x4", max_n=structs) as plan:
        got = plan.scan(dev(x), inclusive=inclusive)
        plan.check()
    assert np.array_equal(host(got), oracle.scan_members(x, inclusive=inclusive))


@pytest.mark.parametrize("inclusive", [False, True])
def test_in_place_and_partial_length(cuda, inclusive):
    x = random_structs(50_000, seed=4)
    d = dev(x)
    canary = d[40_000:].clone()
    with Plan("csdl", "u32x4", max_n=x.shape[0]) as plan:
        plan.scan(d, d, inclusive=inclusive, n=40_000)
        plan.check()
    assert np.array_equal(host(d[:40_000]), oracle.scan_members(x[:40_000], inclusive=inclusive))
    assert torch.equal(d[40_000:], canary)


@pytest.mark.parametrize("inclusive", [False, True])
def test_segmented_struct_scan(cuda, inclusive):
    rng = np.random.default_rng(8)
    lengths = np.concatenate([rng.integers(0, 30, size=2000), rng.integers(1000, 60_000, size=20), [0, 1, 0]])
    rng.shuffle(lengths)
    offs = np.concatenate([[0], np.cumsum(lengths)]).astype(np.uint64)
    n = int(offs[-1])
    x = random_structs(n, seed=9)
    d_off = torch.from_numpy(offs.astype(np.uint32).view(np.int32)).cuda()
    with Plan("csdl", "u32x4", max_n=n) as plan:
        got = plan.scan_segmented(dev(x), d_off, inclusive=inclusive)
        plan.check()
    assert np.array_equal(host(got), oracle.scan_members(x, offs, inclusive))


@pytest.mark.parametrize("split", [1, 2])
@pytest.mark.parametrize("unit,ctas_div", [(1, 1), (4, 1), (1, 2), (4, 2)])
def test_every_launch_configuration_is_exact(cuda, unit, ctas_div, split):
    n = 3_000_001
    x = random_structs(n, seed=unit + 7 * ctas_div + 13 * split)
    with Plan("csdl", "u32x4", max_n=n) as plan:
        if split == 2 and unit == 4:
            # Two threads per row of 16-byte structs with 4-tile units need
            # more shared memory than one CTA has.
            with pytest.raises(GpsError) as e:
                plan.set_generic_config(n, unit, ctas_div, segmented=False, threads_per_row=split)
            assert e.value.status == GPS_ERR_UNSUPPORTED
            return
        plan.set_generic_config(n, unit, ctas_div, segmented=False, threads_per_row=split)
        got = plan.scan(dev(x), inclusive=False)
        plan.check()
    assert np.array_equal(host(got), oracle.scan_members(x, inclusive=False))


def test_large_scan_differences_give_back_the_input(cuda):
    # 2^26 structs (1 GiB in, 1 GiB out): out[i] - out[i-1] == x[i] in every
    # member (mod 2^32) and out[-1] == the member sums.
    n = 1 << 26
    g = torch.Generator(device="cuda").manual_seed(5)
    x = torch.randint(-(1 << 31), 1 << 31, (n, 4), dtype=torch.int32, device="cuda", generator=g)
    with Plan("csdl", "u32x4", max_n=n) as plan:
        out = plan.scan(x, inclusive=True)
        plan.check()
    assert torch.equal(out[1:] - out[:-1], x[1:])  # int32 arithmetic wraps like u32
    assert torch.equal(out[0], x[0])
    sums = (x.to(torch.int64) & 0xFFFFFFFF).sum(dim=0) & 0xFFFFFFFF
    assert torch.equal(out[-1].to(torch.int64) & 0xFFFFFFFF, sums)


def test_graph_replay(cuda):
    n = 700_000
    x = random_structs(n, seed=12)
    want = oracle.scan_members(x, inclusive=False)
    d_in = dev(x)
    out = torch.empty_like(d_in)
    with Plan("csdl", "u32x4", max_n=n) as plan:
        g = torch.cuda.CUDAGraph()
        st = torch.cuda.Stream()
        with torch.cuda.stream(st):
            plan.scan(d_in, out, stream=st)  # warm-up outside the capture
            with torch.cuda.graph(g, stream=st):
                plan.scan(d_in, out, stream=st)
            for _ in range(4):
                out.zero_()
                g.replay()
        st.synchronize()
        plan.check()
    assert np.array_equal(host(out), want)


def test_argument_errors(cuda):
    with pytest.raises(GpsError) as e:
        Plan("rts", "u32x4", max_n=1024)
    assert e.value.status == GPS_ERR_UNSUPPORTED
    with Plan("csdl", "u32x4", max_n=4096) as plan:
        buf = torch.zeros(4096 * 4 + 4, dtype=torch.int32, device="cuda")
        with pytest.raises(GpsError) as e:  # 16-byte structs at a 4-byte offset
            plan.scan_ptr(buf.data_ptr() + 4, buf.data_ptr() + 4, 4096)
        assert e.value.status == GPS_ERR_INVALID_ARGUMENT
        with pytest.raises(GpsError) as e:
            plan.select(buf[:4096 * 4], torch.ones(4096 * 4, dtype=torch.uint8, device="cuda"))
        assert e.value.status == GPS_ERR_UNSUPPORTED
        with pytest.raises(ValueError):
            plan.scan(torch.zeros(6, dtype=torch.int32, device="cuda"))  # not a whole number of structs
