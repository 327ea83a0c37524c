"""Python view of a scan plan (``gps_plan`` in ``include/gps.h``).

A plan corresponds to one constructed reference dispatcher
(``ChainedScanDecoupledLookbackDispatcher(maxSize)`` or
``ReduceThenScanDispatcher(maxSize)``): algorithm, element type and maximum
size are fixed, scratch memory is owned. Data are torch CUDA tensors (or raw
device pointers); every call goes through ``libgps.so``.
"""
from __future__ import annotations

import ctypes

from . import _lib
from ._lib import check, lib

_ALGOS = {"csdl": _lib.ALGO_CSDL, "rts": _lib.ALGO_RTS}
# name -> (gps_dtype, bytes per tensor element, tensor elements per scanned element)
_DTYPES = {"u32": (_lib.DTYPE_U32, 4, 1), "u64": (_lib.DTYPE_U64, 8, 1), "f32": (_lib.DTYPE_F32, 4, 1),
           "f32c": (_lib.DTYPE_F32_COMPENSATED, 4, 1), "u32x4": (_lib.DTYPE_U32X4, 4, 4)}


def _stream_handle(stream) -> int:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class Plan:
    def __init__(self, algo: str = "csdl", dtype: str = "u32", max_n: int = 1 << 20):
        if algo not in _ALGOS:
            raise ValueError(f"algo must be one of {sorted(_ALGOS)}")
        if dtype not in _DTYPES:
            raise ValueError(f"dtype must be one of {sorted(_DTYPES)}")
        self.algo, self.dtype, self.max_n = algo, dtype, int(max_n)
        self.elem_size = _DTYPES[dtype][1]
        # u32x4: a struct of four u32 members; tensors hold n structs as 4n
        # 32-bit words (shape (n, 4)), and sizes count structs.
        self.members = _DTYPES[dtype][2]
        h = ctypes.c_void_p()
        check(lib.gps_plan_create(ctypes.byref(h), _ALGOS[algo], _DTYPES[dtype][0], self.max_n), "gps_plan_create")
        self._h = h

    # -- lifetime
    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._h = None  # never destroyed twice, even if destroy reports an error
            check(lib.gps_plan_destroy(h), "gps_plan_destroy")

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    # -- scans
    def scan_ptr(self, in_ptr: int, out_ptr: int, n: int, inclusive: bool = False, stream=None) -> None:
        kind = _lib.INCLUSIVE if inclusive else _lib.EXCLUSIVE
        check(lib.gps_scan(self._h, kind, ctypes.c_void_p(in_ptr), ctypes.c_void_p(out_ptr), int(n),
                           ctypes.c_void_p(_stream_handle(stream))), "gps_scan")

    def length(self, x) -> int:
        """Number of scanned elements in tensor x (structs for u32x4)."""
        if x.numel() % self.members:
            raise ValueError(f"a {self.dtype} tensor holds a multiple of {self.members} words")
        return x.numel() // self.members

    def scan(self, x, out=None, inclusive: bool = False, n: int | None = None, stream=None):
        """Scan the first n elements of CUDA tensor x into out (allocated if None;
        out may be x for an in-place scan). Bits are taken as unsigned."""
        if x.element_size() != self.elem_size:
            raise TypeError(f"plan is {self.dtype}; tensor has {x.element_size()}-byte elements")
        if not (x.is_cuda and x.is_contiguous()):
            raise ValueError("x must be a contiguous CUDA tensor")
        if out is None:
            import torch
            out = torch.empty_like(x)
        if out.element_size() != self.elem_size or not out.is_contiguous():
            raise ValueError("out must be contiguous with the plan's element size")
        count = self.length(x) if n is None else int(n)
        if count > self.length(x) or count > self.length(out):
            raise ValueError("n exceeds the tensor length")
        self.scan_ptr(x.data_ptr(), out.data_ptr(), count, inclusive, stream)
        return out

    def scan_segmented(self, x, offsets, out=None, inclusive: bool = False, stream=None):
        """Batched scan: independent scans of the segments [offsets[s],
        offsets[s+1]) of CUDA tensor x (offsets: int32/uint32 CUDA tensor of
        num_segments + 1 entries, offsets[0] == 0, offsets[-1] == the number of
        elements, structs for u32x4)."""
        if x.element_size() != self.elem_size or not (x.is_cuda and x.is_contiguous()):
            raise ValueError("x must be a contiguous CUDA tensor with the plan's element size")
        if offsets.element_size() != 4 or not (offsets.is_cuda and offsets.is_contiguous()):
            raise ValueError("offsets must be a contiguous 32-bit CUDA tensor")
        if out is None:
            import torch
            out = torch.empty_like(x)
        kind = _lib.INCLUSIVE if inclusive else _lib.EXCLUSIVE
        check(lib.gps_scan_segmented(self._h, kind, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                     self.length(x), ctypes.c_void_p(offsets.data_ptr()), offsets.numel() - 1,
                                     ctypes.c_void_p(_stream_handle(stream))), "gps_scan_segmented")
        return out

    def select(self, x, flags, out=None, num_selected=None, stream=None):
        """Stream compaction: the elements of CUDA tensor x whose flag byte
        (uint8/bool CUDA tensor, same length) is non-zero, in order, into
        out[:count]; count (int64 CUDA tensor of one element) is written on
        the device. Returns (out, num_selected)."""
        import torch
        if x.element_size() != self.elem_size or not (x.is_cuda and x.is_contiguous()):
            raise ValueError("x must be a contiguous CUDA tensor with the plan's element size")
        if flags.element_size() != 1 or flags.numel() != x.numel() or not (flags.is_cuda and flags.is_contiguous()):
            raise ValueError("flags must be a contiguous one-byte CUDA tensor as long as x")
        if out is None:
            out = torch.empty_like(x)
        if num_selected is None:
            num_selected = torch.zeros(1, dtype=torch.int64, device=x.device)
        check(lib.gps_select_flagged(self._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(flags.data_ptr()),
                                     ctypes.c_void_p(out.data_ptr()), x.numel(),
                                     ctypes.c_void_p(num_selected.data_ptr()), ctypes.c_void_p(_stream_handle(stream))),
              "gps_select_flagged")
        return out, num_selected

    def autotune(self, x, offsets=None, out=None, inclusive: bool = False, stream=None) -> dict:
        """Times the generic kernel's launch configurations on these tensors
        (batched when offsets is given) and keeps the fastest for the size
        class of x.numel(); returns it. out must not be x. Synchronizes; not
        inside a capture."""
        if out is None:
            import torch
            out = torch.empty_like(x)
        kind = _lib.INCLUSIVE if inclusive else _lib.EXCLUSIVE
        unit, div, split = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        off_ptr = ctypes.c_void_p(offsets.data_ptr()) if offsets is not None else ctypes.c_void_p()
        nseg = offsets.numel() - 1 if offsets is not None else 0
        check(lib.gps_plan_autotune(self._h, kind, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                    self.length(x), off_ptr, nseg, ctypes.c_void_p(_stream_handle(stream)),
                                    ctypes.byref(unit), ctypes.byref(div), ctypes.byref(split)), "gps_plan_autotune")
        return {"unit_tiles": unit.value, "ctas_div": div.value, "threads_per_row": split.value}

    def generic_config(self, n: int, segmented: bool = True) -> dict:
        unit, div, split, tuned = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_int()
        check(lib.gps_plan_generic_config(self._h, int(segmented), int(n), ctypes.byref(unit), ctypes.byref(div),
                                          ctypes.byref(split), ctypes.byref(tuned)), "gps_plan_generic_config")
        return {"unit_tiles": unit.value, "ctas_div": div.value, "threads_per_row": split.value,
                "tuned": bool(tuned.value)}

    def set_generic_config(self, n: int, unit_tiles: int, ctas_div: int = 1, segmented: bool = True,
                           threads_per_row: int = 1) -> None:
        check(lib.gps_plan_set_generic_config(self._h, int(segmented), int(n), int(unit_tiles), int(ctas_div),
                                              int(threads_per_row)), "gps_plan_set_generic_config")

    def scan_host(self, h_in: int, h_out: int, n: int, inclusive: bool = False, stream=None) -> None:
        """Scan n elements of a host array (pointers; pinned memory for speed)."""
        kind = _lib.INCLUSIVE if inclusive else _lib.EXCLUSIVE
        check(lib.gps_scan_host(self._h, kind, ctypes.c_void_p(h_in), ctypes.c_void_p(h_out), int(n),
                                ctypes.c_void_p(_stream_handle(stream))), "gps_scan_host")

    # -- status, test modes, geometry
    def check(self, stream=None) -> None:
        check(lib.gps_plan_check(self._h, ctypes.c_void_p(_stream_handle(stream))), "gps_plan_check")

    def check_status(self, stream=None) -> int:
        return lib.gps_plan_check(self._h, ctypes.c_void_p(_stream_handle(stream)))

    def set_wait_budget(self, budget_ns: int) -> None:
        check(lib.gps_plan_set_wait_budget(self._h, int(budget_ns)), "gps_plan_set_wait_budget")

    def set_stall(self, mode: int, period: int = 8, seed: int = 0, delay_ns: int = 0, fallback_polls: int = 0) -> None:
        check(lib.gps_plan_set_stall(self._h, mode, period, seed, delay_ns, fallback_polls), "gps_plan_set_stall")

    def set_fallback(self, fallback_polls: int) -> None:
        """Decoupled fallback: re-reduce a predecessor that shows no progress
        for this many lookback polls (0: off)."""
        check(lib.gps_plan_set_fallback(self._h, int(fallback_polls)), "gps_plan_set_fallback")

    def set_small_max(self, max_n: int) -> None:
        """Largest integer scan run in one CTA (0: always the multi-CTA kernels)."""
        check(lib.gps_plan_set_small_max(self._h, int(max_n)), "gps_plan_set_small_max")

    def set_mid_max(self, max_n: int) -> None:
        """Largest integer chained scan run as one tile per CTA (0: always the
        persistent kernel above the one-CTA size)."""
        check(lib.gps_plan_set_mid_max(self._h, int(max_n)), "gps_plan_set_mid_max")

    def stats(self, stream=None) -> dict:
        s = _lib.LookbackStats()
        check(lib.gps_plan_stats(self._h, ctypes.c_void_p(_stream_handle(stream)), ctypes.byref(s)), "gps_plan_stats")
        return {"polls": s.polls, "fallbacks": s.fallbacks, "inserts": s.inserts, "stalls": s.stalls}

    def geometry(self, n: int) -> dict:
        t, g, l = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        check(lib.gps_plan_geometry(self._h, int(n), ctypes.byref(t), ctypes.byref(g), ctypes.byref(l)),
              "gps_plan_geometry")
        return {"tile_elems": t.value, "grid": g.value, "launches": l.value}

    def scratch_bytes(self) -> int:
        b = ctypes.c_size_t()
        check(lib.gps_plan_scratch_bytes(self._h, ctypes.byref(b)), "gps_plan_scratch_bytes")
        return b.value
