"""The library's FP64 measurements: the DFMA loop's rate (the FP64 roofline
denominator) is positive and below the part's nominal rate, and the
lane-cost loops return times for 1..32 active lanes and refuse others."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


def test_fp64_peak_and_lane_costs(gpu_lib):
    from ctsm_gb300 import _lib
    L = _lib.load()
    L.ctsmg_measure_fp64_tflops.argtypes = [C.POINTER(C.c_double)]
    t = C.c_double()
    _lib.check(L.ctsmg_measure_fp64_tflops(C.byref(t)))
    assert 0.1 < t.value < 200.0
    for fn in ("ctsmg_measure_fp64_lane_cost", "ctsmg_measure_fp64_div_lane_cost"):
        f = getattr(L, fn)
        f.argtypes = [C.c_int32, C.POINTER(C.c_float)]
        ms = {}
        for lanes in (32, 1):
            x = C.c_float()
            _lib.check(f(lanes, C.byref(x)))
            ms[lanes] = x.value
            assert x.value > 0.0
        assert f(0, C.byref(C.c_float())) != 0 and f(33, C.byref(C.c_float())) != 0
