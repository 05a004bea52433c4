"""The shared-reciprocal quotient of ctsm_gb300/csrc/cr_div.cuh on the device
(the special-function unit's reciprocal seed, one Newton step, one
Newton-Markstein correction) against the device's IEEE division a / b over
random and edge-case pairs (whole double range, physical magnitudes, all-ones
significands, zeros, subnormals, infinities, NaN): the same bits except where
a/b lies within 2^-79 |a/b| of a rounding midpoint, where it may be the other
neighbour -- so every quotient is within one ulp and almost none differ -- and
special values exactly as the division.  The reciprocal itself is within
2^-39.8 of 1/b in the fast range."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_device_crdiv_equals_division(gpu_lib):
    from gpu_diag import load, check
    import ctypes as C
    L = load()
    P = C.POINTER(C.c_double)
    r = np.random.Generator(np.random.Philox(11))
    n = 1 << 22
    bits_a = r.integers(0, 2**63, size=n, dtype=np.int64).astype(np.uint64) | \
        (r.integers(0, 2, size=n).astype(np.uint64) << np.uint64(63))
    bits_b = r.integers(0, 2**63, size=n, dtype=np.int64).astype(np.uint64)
    a = bits_a.view(np.float64).copy()
    b = bits_b.view(np.float64).copy()
    q = n // 4
    a[q:2 * q] = r.uniform(-1e6, 1e6, q) * np.exp(r.uniform(-30, 30, q))
    b[q:2 * q] = r.uniform(1e-3, 1e3, q) * np.exp(r.uniform(-30, 30, q))
    ones = (np.uint64(0x000fffffffffffff) ^ r.integers(0, 64, size=q).astype(np.uint64)) | \
        (r.integers(1003, 1044, size=q).astype(np.uint64) << np.uint64(52))
    b[2 * q:3 * q] = ones.view(np.float64)
    a[2 * q:3 * q] = r.uniform(-1e3, 1e3, q)
    special = [0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, 2.2250738585072014e-308, 1.7976931348623157e308, 1.0]
    k = 0
    for x in special:
        for y in special:
            a[3 * q + k], b[3 * q + k] = x, y
            k += 1
    out = np.zeros(3 * n)
    check(L.ctsmg_diag_crdiv(n, a.ctypes.data_as(P), b.ctypes.data_as(P), out.ctypes.data_as(P)))
    ieee, crd, rcp = out.reshape(3, n)
    same = (ieee.view(np.uint64) == crd.view(np.uint64)) | (np.isnan(ieee) & np.isnan(crd))
    ulp = np.abs(ieee.view(np.int64) - crd.view(np.int64))
    assert (same | (ulp <= 1)).all(), (a[~same][:5], b[~same][:5])
    assert (~same).sum() <= 4, (~same).sum()
    ea = (a.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7ff)
    eb = (b.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7ff)
    fast = (ea >= 0x201) & (ea <= 0x5fe) & (eb >= 0x201) & (eb <= 0x5fe)
    special = ~fast
    assert same[special].all()                                   # outside the fast range: the division itself
    with np.errstate(all="ignore"):
        exact = 1.0 / b
    rel = np.abs(rcp[fast] - exact[fast]) / np.abs(exact[fast])
    assert rel.max() < 2.0 ** -39.8, rel.max()
