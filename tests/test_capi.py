"""The C-ABI library on the CPU: it loads, exports every entry point that
include/*.h declares, and rejects bad arguments before touching the GPU."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pytestmark = pytest.mark.usefixtures("built")


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b(gps_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_the_expected_entry_points():
    names = declared_functions()
    for required in ("gps_plan_create", "gps_plan_destroy", "gps_scan", "gps_scan_host", "gps_plan_check"):
        assert required in names


def test_library_exports_every_declared_symbol():
    from gpuprefixsums_gb300 import lib
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_bindings_cover_every_declared_symbol():
    from gpuprefixsums_gb300 import _lib
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert set(declared_functions()) <= bound


def test_status_strings_and_version():
    from gpuprefixsums_gb300 import _lib, lib
    assert lib.gps_version() >= 10000
    for code, name in [(0, b"GPS_OK"), (2, b"GPS_ERR_SIZE_EXCEEDS_PLAN"), (4, b"GPS_ERR_TIMEOUT")]:
        assert lib.gps_status_string(code) == name
    assert lib.gps_status_string(99) == b"GPS_ERR_UNKNOWN"
    assert _lib.GPS_ERR_WRONG_DEVICE == 7


def test_null_plan_is_rejected_without_a_gpu():
    from gpuprefixsums_gb300 import _lib, lib
    assert lib.gps_plan_destroy(None) == _lib.GPS_OK
    assert lib.gps_scan(None, 0, None, None, 10, None) == _lib.GPS_ERR_INVALID_ARGUMENT
    assert b"plan is NULL" in lib.gps_last_error()
    assert lib.gps_scan_host(None, 0, None, None, 10, None) == _lib.GPS_ERR_INVALID_ARGUMENT
    assert lib.gps_plan_check(None, None) == _lib.GPS_ERR_INVALID_ARGUMENT
    assert lib.gps_plan_set_wait_budget(None, 5) == _lib.GPS_ERR_INVALID_ARGUMENT
    assert lib.gps_plan_create(None, 0, 0, 10) == _lib.GPS_ERR_INVALID_ARGUMENT


def test_plan_create_rejects_bad_arguments_before_any_cuda_call():
    from gpuprefixsums_gb300 import _lib, lib
    h = ctypes.c_void_p()
    assert lib.gps_plan_create(ctypes.byref(h), 9, 0, 10) == _lib.GPS_ERR_INVALID_ARGUMENT
    assert lib.gps_plan_create(ctypes.byref(h), 0, 9, 10) == _lib.GPS_ERR_INVALID_ARGUMENT
    assert lib.gps_plan_create(ctypes.byref(h), 0, 0, 0) == _lib.GPS_ERR_INVALID_ARGUMENT
    assert lib.gps_plan_create(ctypes.byref(h), 0, 0, 1 << 60) == _lib.GPS_ERR_INVALID_ARGUMENT
    # Floating-point and struct element types run on chained-scan plans only.
    for dtype in (_lib.DTYPE_F32, _lib.DTYPE_F32_COMPENSATED, _lib.DTYPE_U32X4):
        assert lib.gps_plan_create(ctypes.byref(h), _lib.ALGO_RTS, dtype, 1024) == _lib.GPS_ERR_UNSUPPORTED
    assert h.value is None


def test_plan_setters_reject_a_null_plan_without_a_gpu():
    from gpuprefixsums_gb300 import _lib, lib
    for call in (lambda: lib.gps_plan_set_small_max(None, 0), lambda: lib.gps_plan_set_mid_max(None, 0),
                 lambda: lib.gps_plan_set_fallback(None, 0), lambda: lib.gps_plan_set_wait_budget(None, 1000)):
        assert call() == _lib.GPS_ERR_INVALID_ARGUMENT
        assert b"plan is NULL" in lib.gps_last_error()


def test_compat_selftest_was_built():
    from gpuprefixsums_gb300.build import SELFTEST_BIN
    assert os.access(SELFTEST_BIN, os.X_OK)


def _reference_driver():
    from oracle.build import REFERENCE_SRC
    return os.path.join(REFERENCE_SRC, "GPUPrefixSumsCUDA.cu")


REFERENCE_DRIVER = _reference_driver()


@pytest.mark.skipif(not os.path.exists(REFERENCE_DRIVER), reason="reference checkout not present")
def test_reference_driver_builds_unchanged_against_the_compat_headers(tmp_path):
    """The reference's own main() (GPUPrefixSumsCUDA.cu:14-38) compiles and
    links against include/gps_compat/ and libgps.so with no edit: its quoted
    includes resolve to the compat headers once the file is compiled from a
    directory without the reference headers beside it."""
    import shutil
    import subprocess

    from gpuprefixsums_gb300 import build as B
    src = tmp_path / "GPUPrefixSumsCUDA.cu"
    shutil.copyfile(REFERENCE_DRIVER, src)
    exe = tmp_path / "driver"
    cmd = [B.nvcc_path(), *B.ARCH_FLAGS, "-std=c++17", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "include", "gps_compat"), "-o", str(exe), str(src),
           "-L", B.PKG_DIR, "-lgps", "-Xlinker", "-rpath", "-Xlinker", B.PKG_DIR]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-2000:]
    assert exe.exists()
