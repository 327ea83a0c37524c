"""Build recipe for the oracle (test infrastructure only).

* ``oracle/liboracle.so``: gcc build of ``scan_oracle.c`` (the CPU restatement).
* ``oracle/_ref/``: the reference's own CUDA kernels, compiled from their
  sources under the reference checkout (``GPUPrefixSumsCUDA/*.cuh``) into a
  device-only cubin by ``ref_kernels.cu`` of this folder. Built only where the
  reference checkout exists; elsewhere the previously built files are used.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(ORACLE_DIR, "liboracle.so")
REF_DIR = os.path.join(ORACLE_DIR, "_ref")
REF_CUBIN = os.path.join(REF_DIR, "ref_kernels.cubin")
# The reference's CUDA folder: GPS_REFERENCE_DIR, else the checkout location
# of the build container. This recipe is the only place that names it; where
# neither exists (the GPU machines) the previously built files are used and
# the tests that need the checkout itself skip.
REFERENCE_SRC = os.environ.get("GPS_REFERENCE_DIR") or "/root/reference/GPUPrefixSumsCUDA"


def build_oracle(force: bool = False) -> str:
    src = os.path.join(ORACLE_DIR, "scan_oracle.c")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src):
        return LIB_PATH
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler found for the oracle")
    tmp = LIB_PATH + ".tmp"
    cmd = [cc, "-O2", "-std=c11", "-Wall", "-shared", "-fPIC", "-pthread", "-o", tmp, src, "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_reference_kernels(force: bool = False) -> str | None:
    """Compile the reference's CUDA kernels (unmodified headers) to a cubin."""
    harness = os.path.join(ORACLE_DIR, "ref_kernels.cu")
    if not os.path.isdir(REFERENCE_SRC) or not os.path.exists(harness):
        return REF_CUBIN if os.path.exists(REF_CUBIN) else None
    if not force and os.path.exists(REF_CUBIN) and os.path.getmtime(REF_CUBIN) >= os.path.getmtime(harness):
        return REF_CUBIN
    os.makedirs(REF_DIR, exist_ok=True)
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    tmp = REF_CUBIN + ".tmp"
    cmd = [nvcc, "-cubin", "-gencode=arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
           "-I", REFERENCE_SRC, "-o", tmp, harness]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"reference kernel build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, REF_CUBIN)
    return REF_CUBIN


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference_kernels(force="--force" in sys.argv))
