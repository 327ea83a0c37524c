"""Launches the reference's own CUDA kernels (oracle/_ref/ref_kernels.cubin,
built from the reference's unmodified headers by oracle/build.py) the way the
reference's dispatchers do -- TEST INFRASTRUCTURE ONLY.

Only the chained scan and the reduce-then-scan kernels are launched. The
reference's EmulatedDeadlock kernel is not: its stalled tiles spin on their
own descriptor without any bound (EmulatedDeadlocking.cuh:64-67), and a
stalled tile with no successor never returns.

Buffers passed in are padded to whole 4096-element tiles, because the
reference's Reduce kernel reads the last tile in full (its partial-tile
predicate is inverted, ReduceThenScan.cuh:37) and both paths read and write up
to align4(n) (ScanCommon.cuh:120,201).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUBIN = os.path.join(ROOT, "oracle", "_ref", "ref_kernels.cubin")
PART = 4096  # CSDL_WARPS * 32 * UINT4_PER_THREAD * 4 (Dispatcher.cuh:13-18)


def available() -> bool:
    return os.path.exists(CUBIN)


class RefKernels:
    _NAMES = {
        "csdl_exclusive": "CSDLExclusive",
        "csdl_inclusive": "CSDLInclusive",
        "reduce": "ReduceThenScan6Reduce",
        "spine": "SpineScan",
        "propagate_inclusive": "PropagateInclusive",
        "propagate_exclusive": "PropagateExclusive",
    }

    def __init__(self):
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # primary context current on this thread
        self.cu = ctypes.CDLL("libcuda.so.1")
        cu = self.cu
        self.mod = ctypes.c_void_p()
        self._chk(cu.cuModuleLoad(ctypes.byref(self.mod), CUBIN.encode()), "cuModuleLoad")
        count = ctypes.c_uint()
        self._chk(cu.cuModuleGetFunctionCount(ctypes.byref(count), self.mod), "cuModuleGetFunctionCount")
        funcs = (ctypes.c_void_p * count.value)()
        self._chk(cu.cuModuleEnumerateFunctions(funcs, count, self.mod), "cuModuleEnumerateFunctions")
        names = {}
        for f in funcs:
            name = ctypes.c_char_p()
            self._chk(cu.cuFuncGetName(ctypes.byref(name), ctypes.c_void_p(f)), "cuFuncGetName")
            names[name.value.decode()] = f
        self.fn = {}
        for key, pat in self._NAMES.items():
            hits = [f for n, f in names.items() if pat in n]
            if len(hits) != 1:
                raise RuntimeError(f"reference kernel {pat}: {len(hits)} matches in {sorted(names)}")
            self.fn[key] = ctypes.c_void_p(hits[0])

    @staticmethod
    def _chk(res, what):
        if res != 0:
            raise RuntimeError(f"{what} failed with CUresult {res}")

    def _launch(self, key, grid, block, args, stream):
        holders = []
        for a in args:
            holders.append(ctypes.c_uint64(a) if isinstance(a, Ptr) else ctypes.c_uint32(a))
        params = (ctypes.c_void_p * len(holders))(*[ctypes.addressof(h) for h in holders])
        self._chk(self.cu.cuLaunchKernel(self.fn[key], grid, 1, 1, block, 1, 1, 0, ctypes.c_void_p(stream),
                                         params, None), f"launch {key}")

    def csdl_device(self, buf, n: int, inclusive: bool, tbr=None, bump=None):
        """The reference chained scan in place on the int32 device tensor
        buf[:n], as DispatchKernels{Ex,In}clusive does
        (ChainedScanDecoupledLookbackDispatcher.cuh:172-195): both memsets of
        ClearMemory, then one launch. buf must hold at least align4(n)
        elements (the kernel reads and writes up to there); tbr and bump are
        reused when given. Asynchronous on the current stream."""
        import torch
        aligned = (n + 3) // 4 * 4
        blocks = (aligned + PART - 1) // PART
        if buf.numel() < aligned:
            raise ValueError("buffer smaller than align4(n)")
        if tbr is None or tbr.numel() < blocks:
            tbr = torch.zeros(blocks, dtype=torch.int32, device=buf.device)
        if bump is None:
            bump = torch.zeros(1, dtype=torch.int32, device=buf.device)
        tbr[:blocks].zero_()
        bump.zero_()
        stream = torch.cuda.current_stream().cuda_stream
        key = "csdl_inclusive" if inclusive else "csdl_exclusive"
        self._launch(key, blocks, 256, [Ptr(buf.data_ptr()), Ptr(tbr.data_ptr()), Ptr(bump.data_ptr()), aligned // 4],
                     stream)
        return buf

    def scan(self, algo: str, x: np.ndarray, inclusive: bool) -> np.ndarray:
        """Runs the reference kernel(s) in place on a padded copy of x (uint32)."""
        import torch
        n = x.size
        aligned = (n + 3) // 4 * 4                          # align16() in the dispatchers
        vec = aligned // 4                                  # vectorizeAlignedSize()
        blocks = (aligned + PART - 1) // PART               # divRoundUp(alignedSize, partition)
        buf = torch.zeros(blocks * PART, dtype=torch.int32, device="cuda")
        buf[:n] = torch.from_numpy(x.view(np.int32)).cuda()
        tbr = torch.zeros(blocks, dtype=torch.int32, device="cuda")
        bump = torch.zeros(1, dtype=torch.int32, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        if algo == "csdl":
            key = "csdl_inclusive" if inclusive else "csdl_exclusive"
            self._launch(key, blocks, 256, [Ptr(buf.data_ptr()), Ptr(tbr.data_ptr()), Ptr(bump.data_ptr()), vec],
                         stream)
        elif algo == "rts":
            self._launch("reduce", blocks, 256, [Ptr(buf.data_ptr()), Ptr(tbr.data_ptr()), vec], stream)
            self._launch("spine", 1, 1024, [Ptr(tbr.data_ptr()), blocks], stream)
            key = "propagate_inclusive" if inclusive else "propagate_exclusive"
            self._launch(key, blocks, 256, [Ptr(buf.data_ptr()), Ptr(tbr.data_ptr()), vec], stream)
        else:
            raise ValueError(algo)
        torch.cuda.synchronize()
        return buf[:n].cpu().numpy().view(np.uint32).copy()


class Ptr(int):
    """Marks a 64-bit pointer argument."""
