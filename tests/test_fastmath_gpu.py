"""The column kernels' table-driven log / log10 / exp / pow on the device:
bit-identical to the host build of the same header (every operation is an
explicitly rounded intrinsic), and within a few ulp of the CUDA math
library's functions (CUDA documents 1 ulp for log / log10 / exp and 2 for
pow; the kernels' forms are within 1 / 1.5 / 1 / 1 ulp of the exact values,
tests/test_fastmath_cpu.py)."""
import ctypes as C

import numpy as np
import pytest

import fastmath_host as fh

pytestmark = pytest.mark.gpu


def _ulps(x, ref):
    return np.abs(x - ref) / np.spacing(np.abs(ref))


def test_device_matches_host_and_cuda(gpu_lib, tmp_path):
    from gpu_diag import load, check
    L = load()
    P = C.POINTER(C.c_double)
    r = np.random.Generator(np.random.Philox(5))
    n = 1 << 20
    q = n // 4
    x = np.concatenate([np.exp(r.uniform(np.log(1e-300), np.log(1e300), q)), r.uniform(0.01, 1.0, q),
                        1 + r.uniform(-6e-3, 6e-3, q), r.uniform(1e-3, 5.0, n - 3 * q)])
    y = np.concatenate([r.uniform(-3, 3, q), r.uniform(-15, 30, q), r.uniform(-700, 700, q), r.uniform(-1, 1, n - 3 * q)])
    sp_x = [0.0, -0.0, -1.0, np.inf, np.nan, 5e-324, 1.0, 2.0]
    sp_y = [710.0, -710.0, -745.5, np.inf, np.nan, 1.0, 0.0, 1.0]
    x[:len(sp_x)] = sp_x
    y[:len(sp_y)] = sp_y
    out = np.zeros(8 * n)
    check(L.ctsmg_diag_fastmath(n, x.ctypes.data_as(P), y.ctypes.data_as(P), out.ctypes.data_as(P)))
    dev = out.reshape(8, n)
    host = fh.evaluate(fh.build(tmp_path), x, y)
    # fast range: bit-identical to the host build; outside it the kernels call
    # CUDA's function, so the device result is CUDA's own
    pos = (x >= 2.2250738585072014e-308) & np.isfinite(x)
    for k in range(2):
        np.testing.assert_array_equal(dev[k][pos], host[k][pos])
        np.testing.assert_array_equal(dev[k][~pos], dev[k + 4][~pos])
    fe = np.abs(y) < 704.0
    np.testing.assert_array_equal(dev[2][fe], host[2][fe])
    np.testing.assert_array_equal(dev[2][~fe], dev[6][~fe])
    with np.errstate(all="ignore"):
        t = np.abs(y * np.log(np.where(pos, x, 1.0)))
    fp = pos & (t < 703.9)
    lib = ~pos | (t > 704.1)
    np.testing.assert_array_equal(dev[3][fp], host[3][fp])
    np.testing.assert_array_equal(dev[3][lib], dev[7][lib])
    assert fp.sum() > n // 2
    body = slice(len(sp_x), n)
    finite = np.isfinite(dev[7][body]) & (dev[7][body] != 0) & (np.abs(dev[7][body]) > 1e-300)
    assert _ulps(dev[0][body], dev[4][body]).max() <= 2
    assert _ulps(dev[1][body], dev[5][body]).max() <= 3
    assert _ulps(dev[2][body], dev[6][body]).max() <= 2
    assert _ulps(dev[3][body][finite], dev[7][body][finite]).max() <= 3
    np.testing.assert_array_equal(dev[0][:6], dev[4][:6])
    np.testing.assert_array_equal(dev[2][:5], dev[6][:5])
