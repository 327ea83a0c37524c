"""ctypes binding of the C ABI in ``include/gps.h`` (``libgps.so``).

The library is the only compute path: if it has not been built, importing
this module raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
import os

from .build import LIB_PATH

GPS_OK = 0
GPS_ERR_INVALID_ARGUMENT = 1
GPS_ERR_SIZE_EXCEEDS_PLAN = 2
GPS_ERR_CUDA = 3
GPS_ERR_TIMEOUT = 4
GPS_ERR_UNSUPPORTED = 5
GPS_ERR_OUT_OF_MEMORY = 6
GPS_ERR_WRONG_DEVICE = 7

DTYPE_U32 = 0
DTYPE_U64 = 1
DTYPE_F32 = 2
DTYPE_F32_COMPENSATED = 3
DTYPE_U32X4 = 4
ALGO_CSDL = 0
ALGO_RTS = 1
EXCLUSIVE = 0
INCLUSIVE = 1


class LookbackStats(ctypes.Structure):
    _fields_ = [("polls", ctypes.c_uint64), ("fallbacks", ctypes.c_uint64),
                ("inserts", ctypes.c_uint64), ("stalls", ctypes.c_uint64)]


# (name, restype, argtypes) for every entry point declared in include/gps.h.
_P = ctypes.c_void_p
_U32 = ctypes.c_uint32
_U64 = ctypes.c_uint64
_INT = ctypes.c_int
SIGNATURES = [
    ("gps_version", _INT, []),
    ("gps_status_string", ctypes.c_char_p, [_INT]),
    ("gps_last_error", ctypes.c_char_p, []),
    ("gps_plan_create", _INT, [ctypes.POINTER(_P), _INT, _INT, _U64]),
    ("gps_plan_destroy", _INT, [_P]),
    ("gps_plan_scratch_bytes", _INT, [_P, ctypes.POINTER(ctypes.c_size_t)]),
    ("gps_scan", _INT, [_P, _INT, _P, _P, _U64, _P]),
    ("gps_scan_host", _INT, [_P, _INT, _P, _P, _U64, _P]),
    ("gps_scan_segmented", _INT, [_P, _INT, _P, _P, _U64, _P, _U64, _P]),
    ("gps_select_flagged", _INT, [_P, _P, _P, _P, _U64, _P, _P]),
    ("gps_plan_autotune", _INT, [_P, _INT, _P, _P, _U64, _P, _U64, _P, ctypes.POINTER(_U32), ctypes.POINTER(_U32),
                                 ctypes.POINTER(_U32)]),
    ("gps_plan_set_generic_config", _INT, [_P, _INT, _U64, _U32, _U32, _U32]),
    ("gps_plan_generic_config", _INT, [_P, _INT, _U64, ctypes.POINTER(_U32), ctypes.POINTER(_U32),
                                       ctypes.POINTER(_U32), ctypes.POINTER(_INT)]),
    ("gps_plan_check", _INT, [_P, _P]),
    ("gps_plan_set_wait_budget", _INT, [_P, _U64]),
    ("gps_plan_set_stall", _INT, [_P, _U32, _U32, _U32, _U32, _U32]),
    ("gps_plan_set_fallback", _INT, [_P, _U32]),
    ("gps_plan_set_small_max", _INT, [_P, _U64]),
    ("gps_plan_set_mid_max", _INT, [_P, _U64]),
    ("gps_plan_stats", _INT, [_P, _P, ctypes.POINTER(LookbackStats)]),
    ("gps_plan_geometry", _INT, [_P, _U64, ctypes.POINTER(_U32), ctypes.POINTER(_U32), ctypes.POINTER(_U32)]),
    ("gps_scan_u32_noalloc", _INT, [_INT, _P, _P, _U64, _P]),
]

NOALLOC_MAX_N = 1 << 28  # GPS_NOALLOC_MAX_N in include/gps.h


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    if not os.path.exists(path):
        raise ImportError(
            f"{path} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = load()


class GpsError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        msg = lib.gps_last_error().decode(errors="replace")
        name = lib.gps_status_string(status).decode()
        super().__init__(f"{where}: {name}: {msg}")


def check(status: int, where: str) -> None:
    if status != GPS_OK:
        raise GpsError(status, where)
