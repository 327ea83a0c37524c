"""The device-callable primitives of include/gps_device.cuh (warp, block and
tile scans and reductions) against the oracle, bit-exact, through test
kernels built into _build/libgps_devtest.so."""
import ctypes
import os

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

SEG = {0: 32, 1: 256, 2: 1024, 3: 128 * 16}  # elements per segment by level
OPS = {0: (np.add, 0), 1: (np.maximum, 0), 2: (np.minimum, 0xFFFFFFFF)}


@pytest.fixture(scope="module")
def devtest(cuda):
    from gpuprefixsums_gb300 import build as B
    L = ctypes.CDLL(B.build_device_tests())
    L.gps_devtest_run.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p] * 2 + [ctypes.c_uint64, ctypes.c_int,
                                                                                ctypes.c_int, ctypes.c_void_p]
    return L


def expected(x, seg, op, inclusive, reduce):
    ufunc, ident = OPS[op]
    n = x.size
    pad = (-n) % seg
    xp = np.concatenate([x, np.full(pad, ident, np.uint32)]).reshape(-1, seg).astype(np.uint64)
    if reduce:
        r = ufunc.reduce(xp, axis=1)
        out = np.repeat(r, seg)
    else:
        if op == 0:
            offs = np.arange(0, xp.size + 1, seg, dtype=np.uint64)
            out = oracle.segscan(xp.reshape(-1).astype(np.uint32), offs, inclusive).astype(np.uint64)
        else:
            inc = ufunc.accumulate(xp, axis=1)
            if inclusive:
                out = inc.reshape(-1)
            else:
                exc = np.concatenate([np.full((xp.shape[0], 1), ident, np.uint64), inc[:, :-1]], axis=1)
                out = exc.reshape(-1)
    return (out[:n] & 0xFFFFFFFF).astype(np.uint32)


@pytest.mark.parametrize("level,algo", [(0, 0), (0, 1), (1, 0), (2, 0), (3, 0)])
@pytest.mark.parametrize("op", [0, 1, 2])
@pytest.mark.parametrize("inclusive", [0, 1])
def test_scans(devtest, level, algo, op, inclusive):
    rng = np.random.default_rng(level * 100 + op * 10 + inclusive)
    for n in (1, 31, 1000, 100_003):
        x = rng.integers(0, 2 ** 32, size=n, dtype=np.uint64).astype(np.uint32)
        d_in = torch.from_numpy(x.view(np.int32)).cuda()
        d_out = torch.empty_like(d_in)
        totals = torch.zeros(n // 2048 + 1, dtype=torch.int32, device="cuda")
        rc = devtest.gps_devtest_run(level, op, algo, d_in.data_ptr(), d_out.data_ptr(), n, inclusive, 0,
                                     totals.data_ptr())
        assert rc == 0
        got = d_out.cpu().numpy().view(np.uint32)
        assert np.array_equal(got, expected(x, SEG[level], op, inclusive, False)), (n,)
        if level == 3:  # tile totals
            tot = expected(x, SEG[3], op, True, True)[::SEG[3]]
            assert np.array_equal(totals.cpu().numpy().view(np.uint32)[:tot.size], tot)


@pytest.mark.parametrize("level", [0, 1, 2])
@pytest.mark.parametrize("op", [0, 1, 2])
def test_reductions(devtest, level, op):
    rng = np.random.default_rng(level + 7 * op)
    n = 50_001
    x = rng.integers(0, 2 ** 32, size=n, dtype=np.uint64).astype(np.uint32)
    d_in = torch.from_numpy(x.view(np.int32)).cuda()
    d_out = torch.empty_like(d_in)
    assert devtest.gps_devtest_run(level, op, 0, d_in.data_ptr(), d_out.data_ptr(), n, 1, 1, None) == 0
    assert np.array_equal(d_out.cpu().numpy().view(np.uint32), expected(x, SEG[level], op, True, True))
