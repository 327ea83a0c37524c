"""CPU oracle of the scan library -- TEST INFRASTRUCTURE ONLY.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this package, and only as the checker. The library itself
never imports it.

numpy wrappers over ``liboracle.so`` (``scan_oracle.c``), which restates the
reference's serial validation scan (GPUPrefixSumsD3D12/Shaders/Utility.hlsl:99-125),
its known-answer checks (GPUPrefixSumsCUDA/UtilityKernels.cuh:15-38) and its
seeded input generator (Utility.hlsl:37-66).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .build import LIB_PATH, build_oracle

_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        path = LIB_PATH if os.path.exists(LIB_PATH) else build_oracle()
        L = ctypes.CDLL(path)
        P, U64, I = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int
        for name, args, res in [
            ("oracle_scan_u32", [P, P, U64, I], None),
            ("oracle_scan_u64", [P, P, U64, I], None),
            ("oracle_validate_u32", [P, P, U64, I], U64),
            ("oracle_validate_u64", [P, P, U64, I], U64),
            ("oracle_validate_ones_u32", [P, U64, I], U64),
            ("oracle_init_one_u32", [P, U64], None),
            ("oracle_init_random_taus", [P, U64, ctypes.c_uint32], None),
            ("oracle_segscan_u32", [P, P, P, U64, I], None),
            ("oracle_segscan_u64", [P, P, P, U64, I], None),
            ("oracle_scan_u32_mt", [P, P, U64, I, I], I),
            ("oracle_scan_f32_exact", [P, P, U64, I], None),
            ("oracle_scan_f32_serial", [P, P, U64, I], None),
            ("oracle_select", [P, P, P, U64, I], U64),
            ("oracle_version", [], I),
        ]:
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


def scan(x: np.ndarray, inclusive: bool = False) -> np.ndarray:
    """Serial scan mod 2^w of a uint32 or uint64 array."""
    x = np.ascontiguousarray(x)
    out = np.empty_like(x)
    if x.dtype == np.uint32:
        lib().oracle_scan_u32(_ptr(x), _ptr(out), x.size, int(inclusive))
    elif x.dtype == np.uint64:
        lib().oracle_scan_u64(_ptr(x), _ptr(out), x.size, int(inclusive))
    else:
        raise TypeError(f"unsupported dtype {x.dtype}")
    return out


def validate(x: np.ndarray, result: np.ndarray, inclusive: bool = False) -> int:
    """Number of positions where result differs from the serial scan of x."""
    x = np.ascontiguousarray(x)
    result = np.ascontiguousarray(result)
    if x.dtype != result.dtype or x.size != result.size:
        raise ValueError("input and result must have the same dtype and size")
    fn = lib().oracle_validate_u32 if x.dtype == np.uint32 else lib().oracle_validate_u64
    return int(fn(_ptr(x), _ptr(result), x.size, int(inclusive)))


def validate_ones(result: np.ndarray, inclusive: bool = False) -> int:
    result = np.ascontiguousarray(result, dtype=np.uint32)
    return int(lib().oracle_validate_ones_u32(_ptr(result), result.size, int(inclusive)))


def init_one(n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.uint32)
    lib().oracle_init_one_u32(_ptr(out), n)
    return out


def init_random_taus(n: int, seed: int) -> np.ndarray:
    out = np.empty(n, dtype=np.uint32)
    lib().oracle_init_random_taus(_ptr(out), n, seed & 0xFFFFFFFF)
    return out


def segscan(x: np.ndarray, offsets: np.ndarray, inclusive: bool = False) -> np.ndarray:
    x = np.ascontiguousarray(x)
    offs = np.ascontiguousarray(offsets, dtype=np.uint64)
    out = np.empty_like(x)
    fn = lib().oracle_segscan_u32 if x.dtype == np.uint32 else lib().oracle_segscan_u64
    fn(_ptr(x), _ptr(out), _ptr(offs), offs.size - 1, int(inclusive))
    return out


def scan_mt(x: np.ndarray, out: np.ndarray | None = None, inclusive: bool = False, threads: int = 1) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.uint32)
    if out is None:
        out = np.empty_like(x)
    if lib().oracle_scan_u32_mt(_ptr(x), _ptr(out), x.size, int(inclusive), int(threads)) != 0:
        raise RuntimeError("oracle_scan_u32_mt failed")
    return out


def scan_f32_exact(x: np.ndarray, inclusive: bool = True) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty(x.size, dtype=np.float64)
    lib().oracle_scan_f32_exact(_ptr(x), _ptr(out), x.size, int(inclusive))
    return out


def scan_f32_serial(x: np.ndarray, inclusive: bool = True) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty_like(x)
    lib().oracle_scan_f32_serial(_ptr(x), _ptr(out), x.size, int(inclusive))
    return out


def select(x: np.ndarray, flags: np.ndarray) -> np.ndarray:
    """Stream compaction: the elements of x whose flag byte is non-zero."""
    x = np.ascontiguousarray(x)
    flags = np.ascontiguousarray(flags, dtype=np.uint8)
    out = np.empty_like(x)
    count = lib().oracle_select(_ptr(x), _ptr(flags), _ptr(out), x.size, x.itemsize)
    return out[:count]


def scan_members(x: np.ndarray, offsets: np.ndarray | None = None, inclusive: bool = False) -> np.ndarray:
    """Struct scan: x has shape (n, m), uint32; every member (column) is
    scanned on its own, wrapping mod 2^32, within each segment when offsets
    is given. The reference scans vec4<u32> structs this way, one lookback
    descriptor per member (GPUPrefixSumsWebGPUapis/SharedShaders/
    csdldf_struct.wgsl:144-300, inclusive)."""
    x = np.ascontiguousarray(x, dtype=np.uint32)
    if x.ndim != 2:
        raise ValueError("x must have shape (n, members)")
    cols = [np.ascontiguousarray(x[:, k]) for k in range(x.shape[1])]
    if offsets is None:
        return np.stack([scan(c, inclusive) for c in cols], axis=1)
    return np.stack([segscan(c, offsets, inclusive) for c in cols], axis=1)


def expected_struct_ones(words: int) -> np.ndarray:
    """The reference's known answer for the struct scan of all-ones input:
    word i of the inclusive result is i // 4 + 1
    (GPUPrefixSumsWebGPUapis/SharedShaders/validate.wgsl:51-59)."""
    return (np.arange(words, dtype=np.uint64) // 4 + 1).astype(np.uint32)
