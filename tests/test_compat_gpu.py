"""The drop-in dispatcher classes (include/gps_compat/) run on the GPU.

tests/compat/selftest.cu makes the calls of the reference's driver
(GPUPrefixSumsCUDA/GPUPrefixSumsCUDA.cu:14-38) on the classes with the
reference's names: construct at 2^28; TestAllExclusive / TestAllInclusive
(every size in [4096, 8192] plus 2^26..2^28, all-ones, validated:
ChainedScanDecoupledLookbackDispatcher.cuh:38-114,
ReduceThenScanDispatcher.cuh:36-110, EmulatedDeadlockingDispatcher.cuh:41-77);
BatchTimingInclusive at 2^28 (:116-156) and the CUB comparison
(CubDispatcher.cuh:32-76); destroy. Run with a batch count of 2 so the
timings stay short; the output must read as the reference's does.
"""
import re
import subprocess

import pytest

pytestmark = pytest.mark.gpu


def test_reference_driver_sequence_on_the_compat_classes(cuda):
    from gpuprefixsums_gb300 import build as B
    exe = B.build_compat_selftest()
    res = subprocess.run([exe, "2"], capture_output=True, text=True, timeout=900)
    out = res.stdout
    assert res.returncode == 0, (res.returncode, out[-3000:], res.stderr[-2000:])
    # Five validation runs (CSDL exclusive + inclusive, RTS exclusive +
    # inclusive, forced-stall inclusive), each 4097 sweep sizes + 3 large.
    for name, kind in (("ChainedScanDecoupledLookback", "exclusive"), ("ChainedScanDecoupledLookback", "inclusive"),
                       ("ReduceThenScan", "exclusive"), ("ReduceThenScan", "inclusive"),
                       ("EmulatedDeadlocking", "inclusive")):
        assert f"Beginning GPUPrefixSums {name} {kind} validation test" in out, (name, kind)
    passed = re.findall(r"(\d+)/(\d+) All tests passed\.", out)
    assert passed == [("4100", "4100")] * 5, (passed, out[-3000:])
    assert "Test failed" not in out
    # One keys/sec figure per timed dispatcher: CSDL, RTS, forced stall, CUB.
    speeds = re.findall(r"Estimated speed at 268435456 32-bit elements: ([0-9.E+-]+) keys/sec", out)
    assert len(speeds) == 4, out[-3000:]
    assert all(float(s) > 0 for s in speeds)
