"""The oracle's soil evaporative resistance on a hand-worked column
(SurfaceResistanceMod.F90:330-425, sl_14; :231-303, leepielke_1992)."""
import ctypes as C

import numpy as np

from ctsm_gb300 import abi

LS = -abi.NLEVSNO + 1


def test_sl14_and_leepielke_hand_case():
    from oracle import oracle as orc
    A = {n: np.zeros(abi.field_shape(k, 1, 1, 1), dtype=np.dtype(t)) for (n, k, t, u) in abi.SOILRESIS_FIELDS}
    A["dz"][1 - LS] = 0.02
    A["t_soisno"][1 - LS] = 290.0
    A["h2osoi_liq"][1 - LS] = 0.1 * 0.02 * 1000.0        # vwc 0.1
    A["h2osoi_ice"][1 - LS] = 0.05 * 0.02 * 917.0        # vol_ice 0.05
    A["watsat"][0], A["bsw"][0], A["sucsat"][0], A["watfc"][0] = 0.45, 6.0, 200.0, 0.3
    A["frac_sno"][0], A["frac_h2osfc"][0] = 0.2, 0.1
    io = abi.make_io(abi.SoilResisIO, abi.SOILRESIS_FIELDS, A, 1)
    f = np.array([1], np.int32)
    L = orc.lib()
    for m in (1, 0):
        assert L.oracle_soilevap_resis(C.byref(abi.Bounds(1, 1, 1, 1)), 1, f.ctypes.data_as(C.POINTER(C.c_int32)),
                                       C.byref(io), C.byref(abi.SoilResistanceParams(m, 15.0, 0.8))) == 0
    aird = 0.45 * (200.0 / 1e7) ** (1.0 / 6.0)
    d0 = np.float32(2.12e-5) * (290.0 / np.float64(np.float32(273.15))) ** 1.75
    eps = 0.45 - aird
    dg = eps * d0 * (eps / 0.45) ** (3.0 / 6.0)
    dsl = 15.0 * max(0.001, 0.8 * 0.4 - 0.1) / max(0.001, 0.8 * 0.45 - aird)
    np.testing.assert_allclose(A["dsl"][0], dsl, rtol=1e-13)
    np.testing.assert_allclose(A["soilresis"][0], dsl / (dg * eps * 1e3) + 20.0, rtol=1e-12)
    wx = 0.1 + 0.05
    beta = (1 - 0.3) * 0.25 * (1 - np.cos(np.pi * wx / 0.3)) ** 2 + 0.3
    np.testing.assert_allclose(A["soilbeta"][0], beta, rtol=1e-13)
