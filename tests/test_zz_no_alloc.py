"""gps_scan_u32_noalloc(): the chained scan for callers that may not call
cudaMalloc (a fixed device-memory budget, a context where the allocator must
not be entered, a latency-critical path). Its scratch is a fixed device array
of the library instead of a plan's cudaMalloc'd workspace, so it must give
exactly what gps_scan() gives on a chained-scan u32 plan -- also on a second
call, which finds the array as the first call left it.

Collected last (file name), so that a run stopping at the first failure has
run every other test already; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu


def _noalloc(lib, kind, d_in, d_out, n, stream):
    return lib.gps_scan_u32_noalloc(kind, ctypes.c_void_p(d_in.data_ptr()), ctypes.c_void_p(d_out.data_ptr()),
                                    n, ctypes.c_void_p(stream.cuda_stream))


def test_noalloc_matches_the_plan_scan_on_two_calls_in_a_row(cuda):
    from gpuprefixsums_gb300 import Plan, _lib, lib

    stream = torch.cuda.current_stream()
    cases = [((1 << 22) + 3, _lib.EXCLUSIVE, 11),              # not a tile multiple
             ((1 << 24) + 4096 * 5 + 1, _lib.INCLUSIVE, 12)]   # larger, inclusive
    with Plan("csdl", "u32", max_n=max(c[0] for c in cases)) as plan:
        for n, kind, seed in cases:
            rng = np.random.default_rng(seed)
            x = rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)
            d_in = torch.from_numpy(x.view(np.int32)).cuda()
            want = plan.scan(d_in, inclusive=bool(kind))
            got = torch.full_like(d_in, -1)
            assert _noalloc(lib, kind, d_in, got, n, stream) == _lib.GPS_OK, lib.gps_last_error()
            torch.cuda.synchronize()
            plan.check()
            assert torch.equal(got, want), f"n={n} kind={kind}: differs from gps_scan"
            assert oracle.validate(x, got.cpu().numpy().view(np.uint32), bool(kind)) == 0


def test_noalloc_unaligned_views_and_edge_sizes(cuda):
    # Offset views (element-aligned, not 16-byte aligned) take the ring kernel
    # on the cleared scratch; n = 1 and n = 4095 are under one tile.
    from gpuprefixsums_gb300 import Plan, _lib, lib

    stream = torch.cuda.current_stream()
    with Plan("csdl", "u32", max_n=1 << 20) as plan:
        for n, off_in, off_out, kind in ((1, 0, 0, _lib.EXCLUSIVE), (1, 1, 3, _lib.INCLUSIVE),
                                         (4095, 0, 0, _lib.INCLUSIVE), (4095, 1, 1, _lib.EXCLUSIVE),
                                         (5 * 4096 + 9, 1, 2, _lib.INCLUSIVE), ((1 << 20) - 3, 3, 1, _lib.EXCLUSIVE)):
            rng = np.random.default_rng(n + off_in)
            x = rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)
            big_in = torch.zeros(n + 8, dtype=torch.int32, device="cuda")
            big_in[off_in:off_in + n] = torch.from_numpy(x.view(np.int32)).cuda()
            d_in = big_in[off_in:off_in + n]
            big_out = torch.full((n + 8,), -7, dtype=torch.int32, device="cuda")
            got = big_out[off_out:off_out + n]
            for _ in range(2):  # two calls in a row on the shared scratch
                got.fill_(-1)
                assert _noalloc(lib, kind, d_in, got, n, stream) == _lib.GPS_OK, lib.gps_last_error()
                torch.cuda.synchronize()
                want = plan.scan(d_in.contiguous(), inclusive=bool(kind))
                assert torch.equal(got, want), (n, off_in, off_out, kind)
                assert oracle.validate(x, got.cpu().numpy().view(np.uint32), bool(kind)) == 0
            # nothing written outside [0, n) of the view
            assert int((big_out[:off_out] != -7).sum()) == 0 and int((big_out[off_out + n:] != -7).sum()) == 0
        plan.check()


@pytest.mark.slow
def test_noalloc_at_its_maximum_size(cuda):
    # n = GPS_NOALLOC_MAX_N fills the static descriptor array exactly.
    from gpuprefixsums_gb300 import Plan, _lib, lib

    stream = torch.cuda.current_stream()
    n = _lib.NOALLOC_MAX_N
    gen = torch.Generator(device="cuda").manual_seed(28)
    d_in = torch.randint(-(1 << 31), (1 << 31) - 1, (n,), dtype=torch.int32, device="cuda", generator=gen)
    got = torch.empty_like(d_in)
    with Plan("csdl", "u32", max_n=n) as plan:
        for kind in (_lib.EXCLUSIVE, _lib.INCLUSIVE):
            assert _noalloc(lib, kind, d_in, got, n, stream) == _lib.GPS_OK, lib.gps_last_error()
            want = plan.scan(d_in, inclusive=bool(kind))
            torch.cuda.synchronize()
            plan.check()
            assert torch.equal(got, want), kind
            x = d_in.cpu().numpy().view(np.uint32)
            assert oracle.validate(x, got.cpu().numpy().view(np.uint32), bool(kind)) == 0


def test_noalloc_in_place_and_limit(cuda):
    from gpuprefixsums_gb300 import Plan, _lib, lib

    stream = torch.cuda.current_stream()
    n = 3 * 4096 + 7
    x = torch.randint(-(1 << 31), (1 << 31) - 1, (n,), dtype=torch.int32, device="cuda")
    with Plan("csdl", "u32", max_n=n) as plan:
        want = plan.scan(x, inclusive=False)
    y = x.clone()
    assert _noalloc(lib, _lib.EXCLUSIVE, y, y, n, stream) == _lib.GPS_OK
    torch.cuda.synchronize()
    assert torch.equal(y, want)
    big = _lib.NOALLOC_MAX_N + 1
    st = lib.gps_scan_u32_noalloc(_lib.EXCLUSIVE, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), big,
                                  ctypes.c_void_p(stream.cuda_stream))
    assert st == _lib.GPS_ERR_SIZE_EXCEEDS_PLAN
    assert b"GPS_NOALLOC_MAX_N" in lib.gps_last_error()
