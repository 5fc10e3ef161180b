"""The FP32 FMA probe (nxm_fp32_peak) behind the pair kernel's roofline."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


def test_fp32_peak_probe_reports_plausible_rates():
    from nexusmd_gb300 import engine as E
    L = E.load_library()
    L.nxm_fp32_peak.argtypes = [C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    a, b = C.c_double(), C.c_double()
    assert L.nxm_fp32_peak(0, C.byref(a), C.byref(b)) == 0
    # a GB300 does well above 10 TFLOP/s of FP32 FMA and below 400 in either form
    assert 10.0 < a.value < 400.0 and 10.0 < b.value < 400.0, (a.value, b.value)
    assert L.nxm_fp32_peak(-1, C.byref(a), C.byref(b)) != 0
