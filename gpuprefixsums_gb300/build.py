"""Build recipe for the CUDA scan library ``libgps.so`` (sm_103a only).

Every ``csrc/*.cu`` file is compiled to an object in parallel with nvcc
(``-gencode arch=compute_103a,code=sm_103a``) and linked into
``gpuprefixsums_gb300/libgps.so`` next to this file. Objects are rebuilt only
when a source or header is newer than the library.
"""
from __future__ import annotations

import concurrent.futures
import glob
import os
import shutil
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT_DIR = os.path.dirname(PKG_DIR)
CSRC_DIR = os.path.join(PKG_DIR, "csrc")
INCLUDE_DIR = os.path.join(ROOT_DIR, "include")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libgps.so")
ARCH_FLAGS = ["-gencode=arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    for key in ("CUDA_HOME", "CUDA_PATH"):
        if os.environ.get(key):
            return os.environ[key]
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def nvcc_path() -> str:
    return os.path.join(cuda_home(), "bin", "nvcc")


def common_flags() -> list[str]:
    return ARCH_FLAGS + [
        "-O3",
        "-lineinfo",
        "-std=c++17",
        "-Xcompiler", "-fPIC",
        "-Xcompiler", "-Wall",
        "--expt-relaxed-constexpr",
        "-I", INCLUDE_DIR,
        "-I", CSRC_DIR,
    ]


def _newest_input_mtime() -> float:
    """Newest source the library is built from: every file under csrc/ and
    include/ (the kernels include include/gps_device.cuh), and this recipe."""
    files = [f for d in (CSRC_DIR, INCLUDE_DIR) for f in glob.glob(os.path.join(d, "**", "*"), recursive=True)
             if os.path.isfile(f)]
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


def _compile(src: str, obj: str, extra: list[str]) -> None:
    cmd = [nvcc_path(), *common_flags(), *extra, "-c", src, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{res.stdout}\n{res.stderr}")


def build_library(force: bool = False, ptxas_verbose: bool = False) -> str:
    """Compile and link libgps.so; returns its path."""
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= _newest_input_mtime():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC_DIR, "*.cu")))
    if not sources:
        raise RuntimeError(f"no CUDA sources under {CSRC_DIR}")
    extra = ["-Xptxas", "-v"] if ptxas_verbose else []
    objects = [os.path.join(BUILD_DIR, os.path.basename(s)[:-3] + ".o") for s in sources]
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(sources))) as pool:
        list(pool.map(lambda so: _compile(so[0], so[1], extra), zip(sources, objects)))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc_path(), *ARCH_FLAGS, "-shared", "-cudart", "shared", "-o", tmp, *objects,
           "-Xlinker", "-rpath", "-Xlinker", os.path.join(cuda_home(), "lib64")]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link of libgps.so failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


CUB_SRC = os.path.join(CSRC_DIR, "compare", "cub_scan.cu")
CUB_LIB = os.path.join(PKG_DIR, "libgps_cub.so")


def build_cub_compare(force: bool = False) -> str:
    """Build libgps_cub.so, CUB's DeviceScan for sm_103a: the benchmark's
    comparison bar, kept apart from libgps.so."""
    if not force and os.path.exists(CUB_LIB) and os.path.getmtime(CUB_LIB) >= os.path.getmtime(CUB_SRC):
        return CUB_LIB
    tmp = CUB_LIB + ".tmp"
    cmd = [nvcc_path(), *ARCH_FLAGS, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
           "-cudart", "shared", "-o", tmp, CUB_SRC,
           "-Xlinker", "-rpath", "-Xlinker", os.path.join(cuda_home(), "lib64")]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"CUB comparison build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, CUB_LIB)
    return CUB_LIB


SELFTEST_SRC = os.path.join(ROOT_DIR, "tests", "compat", "selftest.cu")
SELFTEST_BIN = os.path.join(BUILD_DIR, "compat_selftest")


def build_compat_selftest(force: bool = False) -> str:
    """Build the program that drives the drop-in dispatcher classes of
    include/gps_compat/ the way the reference's driver does."""
    lib = build_library()
    deps = [SELFTEST_SRC, lib] + glob.glob(os.path.join(INCLUDE_DIR, "gps_compat", "*"))
    if not force and os.path.exists(SELFTEST_BIN) and \
            os.path.getmtime(SELFTEST_BIN) >= max(os.path.getmtime(d) for d in deps):
        return SELFTEST_BIN
    os.makedirs(BUILD_DIR, exist_ok=True)
    cmd = [nvcc_path(), *ARCH_FLAGS, "-O2", "-std=c++17",
           "-I", INCLUDE_DIR, "-I", os.path.join(INCLUDE_DIR, "gps_compat"),
           "-o", SELFTEST_BIN, SELFTEST_SRC, "-L", PKG_DIR, "-lgps",
           "-Xlinker", "-rpath", "-Xlinker", PKG_DIR]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compat self-test build failed:\n{res.stdout}\n{res.stderr}")
    return SELFTEST_BIN


DEVTEST_SRC = os.path.join(os.path.dirname(PKG_DIR), "tests", "device", "primitives_test.cu")
DEVTEST_LIB = os.path.join(BUILD_DIR, "libgps_devtest.so")


def build_device_tests(force: bool = False) -> str:
    """Build the test kernels of include/gps_device.cuh (the device-callable
    primitives) into _build/libgps_devtest.so."""
    deps = [DEVTEST_SRC, os.path.join(INCLUDE_DIR, "gps_device.cuh")]
    if not force and os.path.exists(DEVTEST_LIB) and \
            os.path.getmtime(DEVTEST_LIB) >= max(os.path.getmtime(d) for d in deps):
        return DEVTEST_LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = DEVTEST_LIB + ".tmp"
    cmd = [nvcc_path(), *ARCH_FLAGS, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-cudart", "shared",
           "-I", INCLUDE_DIR, "-o", tmp, DEVTEST_SRC,
           "-Xlinker", "-rpath", "-Xlinker", os.path.join(cuda_home(), "lib64")]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"device primitive tests build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, DEVTEST_LIB)
    return DEVTEST_LIB


if __name__ == "__main__":
    print(build_library(force=True))
    print(build_compat_selftest(force=True))
