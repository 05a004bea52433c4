"""The integer-pipe comparisons, min and max of ctsm_gb300/csrc/fcmp.cuh
against the device's FP64 instructions over random and edge-case pairs
(signed zeros, subnormals, infinities, NaN of either sign, equal operands,
the literals the soil kernels compare against): every comparison gives the
same truth value, min / max the same value (a NaN operand yields the other
operand, as fmin / fmax), the forms against a positive or negative constant
or zero agree likewise, and fm::i2d builds (double)k exactly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pairs():
    r = np.random.Generator(np.random.Philox(12))
    special = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, -np.nan, 5e-324, -5e-324,
                        2.2250738585072014e-308, -2.2250738585072014e-308, 1.7976931348623157e308,
                        -1.7976931348623157e308, 273.15, np.nextafter(273.15, 400.0), np.nextafter(273.15, 0.0),
                        1e-6, 0.01, 156.0, 1e-7])
    sa, sb = np.meshgrid(special, special)
    n = 1 << 20
    bits_a = r.integers(0, 2**63, size=n, dtype=np.int64).astype(np.uint64) | \
        (r.integers(0, 2, size=n).astype(np.uint64) << np.uint64(63))
    bits_b = r.integers(0, 2**63, size=n, dtype=np.int64).astype(np.uint64) | \
        (r.integers(0, 2, size=n).astype(np.uint64) << np.uint64(63))
    a = bits_a.view(np.float64).copy()
    b = bits_b.view(np.float64).copy()
    q = n // 4
    a[:q] = r.uniform(-300.0, 300.0, q)
    b[:q] = r.choice(special[np.isfinite(special)], q)
    b[q:2 * q] = a[q:2 * q]                                     # equal operands
    a = np.concatenate([sa.ravel(), a])
    b = np.concatenate([sb.ravel(), b])
    return a, b


def test_integer_pipe_comparisons_match_fp64(gpu_lib):
    from gpu_diag import load, check
    import ctypes as C
    L = load()
    P = C.POINTER(C.c_double)
    a, b = _pairs()
    n = a.size
    out = np.zeros(32 * n)
    check(L.ctsmg_diag_fcmp(n, a.ctypes.data_as(P), b.ctypes.data_as(P), out.ctypes.data_as(P)))
    o = out.reshape(32, n)
    for k in range(7):
        assert np.array_equal(o[k], o[8 + k]), (k, a[o[k] != o[8 + k]][:4], b[o[k] != o[8 + k]][:4])
    with np.errstate(invalid="ignore"):
        np.testing.assert_array_equal(o[0], (a < b).astype(float))
        np.testing.assert_array_equal(o[15], (np.abs(a) >= np.abs(b)).astype(float))
    for ieee, mine in ((o[16], o[18]), (o[17], o[19])):
        same = (ieee == mine) | (np.isnan(ieee) & np.isnan(mine))
        assert same.all(), (a[~same][:4], b[~same][:4])
    k = np.arange(n) - n // 2
    np.testing.assert_array_equal(o[20], k.astype(np.float64))
    # the constant forms (a positive or negative second operand, and zero)
    with np.errstate(invalid="ignore"):
        pos, neg = b > 0, b < 0
        np.testing.assert_array_equal(o[21][pos], (a < b)[pos]); np.testing.assert_array_equal(o[21][neg], (a < b)[neg])
        np.testing.assert_array_equal(o[23][pos], (a > b)[pos]); np.testing.assert_array_equal(o[23][neg], (a > b)[neg])
        np.testing.assert_array_equal(o[22][pos], (a <= b)[pos]); np.testing.assert_array_equal(o[24][pos], (a >= b)[pos])
        for row, ref in ((25, a < 0), (26, a <= 0), (27, a > 0), (28, a >= 0)):
            np.testing.assert_array_equal(o[row], ref.astype(float))
    # min / max against the device's fmin / fmax (numpy's fmin returns NaN for
    # a signalling-NaN operand on some hosts; the device's returns the other)
    for mine, ieee in ((o[29], o[16]), (o[30], o[17])):
        same = (mine[pos] == ieee[pos]) | (np.isnan(mine[pos]) & np.isnan(ieee[pos]))
        assert same.all(), (a[pos][~same][:4], b[pos][~same][:4], mine[pos][~same][:4], ieee[pos][~same][:4])
    same = (o[31] == o[7]) | (np.isnan(o[31]) & np.isnan(o[7]))
    assert same.all(), (a[~same][:4], o[31][~same][:4], o[7][~same][:4])
