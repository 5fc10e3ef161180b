"""bench.py's hardware probes (bench_probe.cu, libnxm_probe.so): the FP32 FMA
peak behind the pair kernel's roofline and the shared-memory atomic rates."""
import ctypes as C
import os
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _probe():
    sys.path.insert(0, ROOT)
    import bench
    return bench.probe_library()


def test_fp32_peak_probe_reports_plausible_rates():
    L = _probe()
    a, b = C.c_double(), C.c_double()
    assert L.nxm_probe_fp32_peak(0, C.byref(a), C.byref(b)) == 0
    # a GB300 does well above 10 TFLOP/s of FP32 FMA and below 400 in either form
    assert 10.0 < a.value < 400.0 and 10.0 < b.value < 400.0, (a.value, b.value)
    assert L.nxm_probe_fp32_peak(-1, C.byref(a), C.byref(b)) != 0


def test_shared_atomics_probe_reports_plausible_rates():
    L = _probe()
    a, b = C.c_double(), C.c_double()
    assert L.nxm_probe_shared_atomics(0, C.byref(a), C.byref(b)) == 0
    # per SM per clock: at most one warp's 32 lanes, and not zero
    assert 0.01 < a.value < 64.0 and 0.01 < b.value < 64.0, (a.value, b.value)
