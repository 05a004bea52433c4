"""The device Ci root finder (a single-evaluation-site state machine) visits
exactly the points the oracle's nested hybrid -> brent visits
(PhotosynthesisMod.F90:2251-2485), in the same order, on functions that take
every exit: exact zeros, the secant tolerance, |f| <= 1e-4, Brent's
convergence and its 20-iteration limit, and the 40-iteration limit with the
re-evaluation at the minimum.  Both sides are compiled on the host with the
same flags."""
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CAP = 256


@pytest.fixture(scope="module")
def libs():
    from oracle import oracle as orc
    O = orc.lib()
    d = tempfile.mkdtemp(prefix="rf_")
    so = os.path.join(d, "librf.so")
    subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-std=c++17",
                           "-I", os.path.join(ROOT, "ctsm_gb300", "csrc"), "-I", os.path.join(ROOT, "oracle"),
                           os.path.join(ROOT, "tests", "rootfind_harness.cpp"), "-o", so])
    H = C.CDLL(so)
    sig = [C.c_int, C.POINTER(C.c_double), C.c_double, C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_int)]
    H.rf_trace.argtypes = sig
    O.oracle_rootfind_trace.argtypes = sig
    return O, H


def _trace(fn, k, prm, x0):
    p = np.ascontiguousarray(prm, dtype=np.float64)
    xs = np.zeros(CAP)
    nb = C.c_int()
    n = fn(k, p.ctypes.data_as(C.POINTER(C.c_double)), x0, xs.ctypes.data_as(C.POINTER(C.c_double)), CAP, C.byref(nb))
    return xs[:min(n, CAP)], n, nb.value


CASES = [(0, [250.0, 0, 0, 0], 280.0), (0, [280.0, 0, 0, 0], 280.0), (1, [100.0, 5.0, 0, 0], 160.0),
         (2, [150.0, 1000.0, 1.0, 0], 280.0), (3, [199.0, 0, 0, 0], 200.0), (4, [200.0, 3.0, 0, 0], 300.0),
         (4, [200.0, 0.01, 0, 0], 300.0)]


@pytest.mark.parametrize("k,prm,x0", CASES)
def test_trace_matches_oracle(libs, k, prm, x0):
    O, H = libs
    a, na, nba = _trace(O.oracle_rootfind_trace, k, prm, x0)
    b, nb, nbb = _trace(H.rf_trace, k, prm, x0)
    assert na == nb and nba == nbb
    np.testing.assert_array_equal(a, b)


def test_random_functions_and_paths(libs):
    O, H = libs
    r = np.random.Generator(np.random.Philox(17))
    lengths = []
    for i in range(3000):
        prm = [r.uniform(-1, 1) * 10 ** r.uniform(-4, 0), r.uniform(50, 400), r.uniform(-2, 2), r.uniform(0.5, 50)]
        x0 = r.uniform(20, 600)
        a, na, nba = _trace(O.oracle_rootfind_trace, 5, prm, x0)
        b, nb, nbb = _trace(H.rf_trace, 5, prm, x0)
        assert na == nb and nba == nbb, i
        np.testing.assert_array_equal(a, b)
        lengths.append(na)
    lengths = np.array(lengths)
    # the sample reaches short exits, Brent runs and the iteration limit
    assert lengths.min() <= 3 and lengths.max() >= 42 and len(np.unique(lengths)) > 15
