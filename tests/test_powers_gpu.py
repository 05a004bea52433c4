"""The soil step evaluates the two powers with a constant base --
10^(-e_ice icefrac) (IceImpedance) and tkwat^(fl ws) tkice^((1-fl) ws)
(Johansen's saturated conductivity) -- as exp of a double-double exponent.
Checked here against CUDA's own pow on the device and, where mpmath is
available, against the exact values: within 2 ulp of the exact power, and
within 4 ulp of the pow-based expression (whose own error is up to ~2 ulp per
pow)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ulps(x, ref):
    return np.abs(x - ref) / np.spacing(np.abs(ref))


def test_constant_base_powers(gpu_lib):
    from gpu_diag import load, check
    L = load()
    P = C.POINTER(C.c_double)
    r = np.random.Generator(np.random.Philox(3))
    n = 200000
    x = np.concatenate([-6.0 * r.uniform(0, 1, n - 4), [0.0, -0.0, -6.0, -1e-300]])
    ws = r.uniform(0.25, 0.95, n)
    fl = r.uniform(0, 1, n)
    a = np.ascontiguousarray(fl * ws)
    b = np.ascontiguousarray((1.0 - fl) * ws)
    out = np.zeros(4 * n)
    check(L.ctsmg_diag_powers(n, x.ctypes.data_as(P), x.ctypes.data_as(P), out.ctypes.data_as(P)))
    p10, e10 = out.reshape(4, n)[:2].copy()
    check(L.ctsmg_diag_powers(n, a.ctypes.data_as(P), b.ctypes.data_as(P), out.ctypes.data_as(P)))
    ptk, etk = out.reshape(4, n)[2:].copy()
    assert np.all(e10[-4:-2] == 1.0)
    assert _ulps(e10, p10).max() <= 4 and _ulps(etk, ptk).max() <= 4
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    idx = r.choice(n, 2000, replace=False)
    t10 = np.array([float(mp.power(10, mp.mpf(float(x[i])))) for i in idx])
    ttk = np.array([float(mp.power(mp.mpf(0.57), mp.mpf(float(a[i]))) * mp.power(mp.mpf(2.29), mp.mpf(float(b[i]))))
                    for i in idx])
    assert _ulps(e10[idx], t10).max() <= 2
    assert _ulps(etk[idx], ttk).max() <= 2
