"""The column kernels' table-driven log, log10, exp and pow
(ctsm_gb300/csrc/fastmath.cuh; Tang 1989 / 1990) against 40-digit
references: within 1 ulp for log, exp and pow (CUDA documents 1, 1 and 2 ulp
for its own) and 1.5 ulp for log10; C99 special values where the fast range
ends; and the breakpoint tables are the generator's output."""
import os
import subprocess
import sys

import numpy as np
import pytest

import fastmath_host as fh

mp = pytest.importorskip("mpmath")


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    return fh.build(tmp_path_factory.mktemp("fm"))


def _ulps(v, ref):
    return np.array([float(abs(mp.mpf(float(a)) - r) / mp.mpf(np.spacing(abs(float(r))))) for a, r in zip(v, ref)])


def _samples():
    r = np.random.Generator(np.random.Philox(11))
    n = 1500
    x = np.concatenate([np.exp(r.uniform(np.log(1e-300), np.log(1e300), n)), 1 + r.uniform(-6e-3, 6e-3, n),
                        r.uniform(0.01, 1.0, n), 1.0 + np.arange(1, 256) / 256.0])
    y = np.concatenate([r.uniform(-700, 700, n), r.uniform(-1, 1, n), r.uniform(-15, 30, n), r.uniform(-3, 3, 255)])
    return x, y


def test_accuracy_against_exact(lib):
    mp.mp.dps = 40
    x, y = _samples()
    out = fh.evaluate(lib, x, y)
    xs = [mp.mpf(float(v)) for v in x]
    assert _ulps(out[0], [mp.log(v) for v in xs]).max() <= 1.0
    assert _ulps(out[1], [mp.log10(v) for v in xs]).max() <= 1.5
    assert _ulps(out[2], [mp.exp(mp.mpf(float(v))) for v in y]).max() <= 1.0
    # pow: soil-water arguments (saturation^exponent) and general ones kept in range
    py = np.clip(y, -600.0 / np.maximum(np.abs(np.log(x)), 1e-300), 600.0 / np.maximum(np.abs(np.log(x)), 1e-300))
    out = fh.evaluate(lib, x, py)
    assert _ulps(out[3], [mp.power(a, mp.mpf(float(b))) for a, b in zip(xs, py)]).max() <= 1.0


def test_exact_cases_and_special_values(lib):
    x = np.array([1.0, 2.0, 0.5, 1024.0, 0.0, -0.0, -1.0, np.inf, np.nan, 5e-324, 2.2e-308, 1e308, 0.3, 0.3])
    y = np.array([0.0, 1.0, -1.0, 0.5, 710.0, -710.0, -745.5, np.inf, -np.inf, np.nan, 704.0, -704.0, 3.0, -0.0])
    out = fh.evaluate(lib, x, y)
    with np.errstate(all="ignore"):
        ref_log, ref_exp, ref_pow = np.log(x), np.exp(y), np.power(x, y)
    assert out[0][0] == 0.0 and out[0][1] == np.log(2.0) and out[0][2] == -np.log(2.0)
    np.testing.assert_array_equal(out[0][4:10], ref_log[4:10])      # zero, negative, inf, nan, subnormal
    np.testing.assert_array_equal(out[2][4:10], ref_exp[4:10])      # overflow, underflow, inf, nan
    assert out[2][0] == 1.0 and out[3][0] == 1.0 and out[3][1] == 2.0 and out[3][2] == 2.0
    np.testing.assert_array_equal(out[3][4:9], ref_pow[4:9])
    assert out[3][13] == 1.0 and out[1][3] == pytest.approx(np.log10(1024.0), rel=2.3e-16)


def test_tables_are_the_generators_output():
    here = os.path.dirname(os.path.abspath(__file__))
    csrc = os.path.join(os.path.dirname(here), "ctsm_gb300", "csrc")
    gen = subprocess.run([sys.executable, os.path.join(csrc, "gen_fastmath_tables.py")], check=True,
                         capture_output=True, text=True).stdout
    with open(os.path.join(csrc, "fastmath_tables.h")) as f:
        assert f.read() == gen
