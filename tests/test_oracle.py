"""The oracle against the reference's known answers and against independent
restatements (CPU only)."""
import fractions

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.usefixtures("built")


def py_scan(x, inclusive, mod):
    out, s = [], 0
    for v in x:
        if inclusive:
            s = (s + int(v)) % mod
            out.append(s)
        else:
            out.append(s)
            s = (s + int(v)) % mod
    return out


@pytest.mark.parametrize("inclusive", [False, True])
def test_all_ones_every_size_of_the_reference_sweep(inclusive):
    # ChainedScanDecoupledLookbackDispatcher.cuh:48-59 / UtilityKernels.cuh:22-38:
    # every n in [4096, 8192], all-ones input, inclusive = i + 1, exclusive = i.
    for n in range(4096, 8193):
        out = oracle.scan(oracle.init_one(n), inclusive)
        assert oracle.validate_ones(out, inclusive) == 0, n


@pytest.mark.parametrize("inclusive", [False, True])
def test_all_ones_large_sizes(inclusive):
    # The reference's intended large checks, 2^26..2^28 (its loop passes the
    # exponent instead of the size; these use the size).
    for k in (26, 27, 28):
        n = 1 << k
        out = oracle.scan(oracle.init_one(n), inclusive)
        assert oracle.validate_ones(out, inclusive) == 0
        assert int(out[-1]) == ((n if inclusive else n - 1) & 0xFFFFFFFF)


@pytest.mark.parametrize("dtype,mod", [(np.uint32, 1 << 32), (np.uint64, 1 << 64)])
@pytest.mark.parametrize("inclusive", [False, True])
def test_serial_scan_matches_python_restatement(dtype, mod, inclusive):
    rng = np.random.default_rng(7)
    for n in (0, 1, 2, 3, 17, 1000):
        x = rng.integers(0, np.iinfo(dtype).max, size=n, dtype=dtype, endpoint=True)
        assert oracle.scan(x, inclusive).tolist() == py_scan(x.tolist(), inclusive, mod)


@pytest.mark.parametrize("inclusive", [False, True])
def test_serial_scan_matches_numpy_cumsum_with_wraparound(inclusive):
    rng = np.random.default_rng(11)
    x = rng.integers(0, 1 << 32, size=1 << 20, dtype=np.uint64).astype(np.uint32)
    ref = np.cumsum(x, dtype=np.uint32)
    if not inclusive:
        ref = np.concatenate([[0], ref[:-1]]).astype(np.uint32)
    assert np.array_equal(oracle.scan(x, inclusive), ref)


def test_validate_detects_a_planted_mistake():
    x = np.arange(1000, dtype=np.uint32)
    good = oracle.scan(x, True)
    assert oracle.validate(x, good, True) == 0
    bad = good.copy()
    bad[637] += 1
    assert oracle.validate(x, bad, True) == 1
    bad[999] ^= 4
    assert oracle.validate(x, bad, True) == 2


def py_taus(n, seed):
    # Utility.hlsl:37-66, restated a second time in Python.
    m = 0xFFFFFFFF
    out = [0] * n
    for i in range(min(n, 65536)):
        z1 = ((i << 2) * seed) & m
        z2 = (((i << 2) + 1) * seed) & m
        z3 = (((i << 2) + 2) * seed) & m
        z4 = (((i << 2) + 3) * seed) & m
        z1 = (((z1 & 4294967294) << 12) & m) ^ ((((z1 << 13) & m) ^ z1) >> 19)
        z2 = (((z2 & 4294967288) << 4) & m) ^ ((((z2 << 2) & m) ^ z2) >> 25)
        z3 = (((z3 & 4294967280) << 17) & m) ^ ((((z3 << 3) & m) ^ z3) >> 11)
        z4 = (z4 * 1664525 + 1013904223) & m
        t = (z1 ^ z2 ^ z3 ^ z4) & 1023
        for j in range(i, n, 65536):
            out[j] = t
    return out


@pytest.mark.parametrize("seed", [1, 5, 0xDEADBEEF])
def test_tausworthe_input_generator(seed):
    n = 70000
    got = oracle.init_random_taus(n, seed)
    assert got.tolist() == py_taus(n, seed)
    assert got.max() <= 1023


@pytest.mark.parametrize("threads", [1, 2, 3, 7, 16])
@pytest.mark.parametrize("inclusive", [False, True])
def test_threaded_cpu_scan_equals_serial(threads, inclusive):
    rng = np.random.default_rng(threads)
    for n in (0, 1, 5, 4097, 1 << 18):
        x = rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)
        ref = oracle.scan(x, inclusive)
        assert np.array_equal(oracle.scan_mt(x, inclusive=inclusive, threads=threads), ref)
        y = x.copy()
        oracle.scan_mt(y, out=y, inclusive=inclusive, threads=threads)  # in place
        assert np.array_equal(y, ref)


@pytest.mark.parametrize("inclusive", [False, True])
def test_segmented_scan(inclusive):
    rng = np.random.default_rng(3)
    lens = rng.integers(0, 50, size=40)
    offs = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    x = rng.integers(0, 1 << 32, size=int(offs[-1]), dtype=np.uint64).astype(np.uint32)
    got = oracle.segscan(x, offs, inclusive)
    for s in range(len(lens)):
        b, e = int(offs[s]), int(offs[s + 1])
        assert got[b:e].tolist() == py_scan(x[b:e].tolist(), inclusive, 1 << 32)


def test_exact_fp32_prefix_is_correctly_rounded():
    rng = np.random.default_rng(5)
    mags = 10.0 ** rng.uniform(-8, 8, size=3000)
    x = (mags * rng.choice([-1.0, 1.0], size=3000)).astype(np.float32)
    x[::97] = np.float32(1e-45)  # subnormals
    x[5] = np.float32(3.4e38)
    x[6] = np.float32(-3.4e38)
    got = oracle.scan_f32_exact(x, inclusive=True)
    acc = fractions.Fraction(0)
    for i, v in enumerate(x.tolist()):
        acc += fractions.Fraction(v)
        assert got[i] == float(acc), i
    exc = oracle.scan_f32_exact(x[:10], inclusive=False)
    assert exc[0] == 0.0 and exc[1] == float(x[0])


def test_select_matches_boolean_indexing():
    rng = np.random.default_rng(9)
    for dtype in (np.uint32, np.uint64):
        x = rng.integers(0, 2 ** 31, size=10_001).astype(dtype)
        flags = (rng.random(x.size) < 0.3).astype(np.uint8) * rng.integers(1, 256, size=x.size).astype(np.uint8)
        assert np.array_equal(oracle.select(x, flags), x[flags != 0])
    assert oracle.select(np.zeros(0, np.uint32), np.zeros(0, np.uint8)).size == 0


@pytest.mark.parametrize("inclusive", [False, True])
def test_struct_scan_scans_each_member(inclusive):
    rng = np.random.default_rng(21)
    x = rng.integers(0, 1 << 32, size=(777, 4), dtype=np.uint64).astype(np.uint32)
    got = oracle.scan_members(x, inclusive=inclusive)
    for k in range(4):
        assert got[:, k].tolist() == py_scan(x[:, k].tolist(), inclusive, 1 << 32)
    lens = rng.integers(0, 60, size=25)
    offs = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    y = x[: int(offs[-1])]
    seg = oracle.scan_members(y, offs, inclusive)
    for s in range(len(lens)):
        b, e = int(offs[s]), int(offs[s + 1])
        for k in range(4):
            assert seg[b:e, k].tolist() == py_scan(y[b:e, k].tolist(), inclusive, 1 << 32)


@pytest.mark.parametrize("structs", [1, 1024, 4096 + 3, 1 << 16])
def test_struct_scan_known_answer_of_all_ones(structs):
    # Inclusive scan of all-ones structs: word i of the result is i // 4 + 1.
    got = oracle.scan_members(np.ones((structs, 4), np.uint32), inclusive=True)
    assert np.array_equal(got.reshape(-1), oracle.expected_struct_ones(4 * structs))
