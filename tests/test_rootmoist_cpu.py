"""The oracle's root moisture stress (SoilMoistStressMod.F90:70-114, 171-217,
312-435) on a hand-worked two-patch column: every branch of the level loop
(liquid, no liquid, too cold, ice-bounded porosity) and the normalisation."""
import ctypes as C

import numpy as np

from ctsm_gb300 import abi, canopy_inputs, full_inputs as fi

LS = -abi.NLEVSNO + 1


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def test_root_moist_stress_hand_case():
    from oracle import oracle as orc
    L = orc.lib()
    L.oracle_set_canopy_params(C.byref(canopy_inputs.make_params()), C.byref(canopy_inputs.make_pftcon()), 1, 40)
    A, npatch, ngrid, rootr = fi.full_state(1, seed=3, npatch_max=1)
    A = {k: v for k, v in A.items()}
    npatch = 2
    A["patch_column"] = np.array([1, 1], dtype=np.int32)
    A["itype"] = np.array([1, 1], dtype=np.int32)
    fr = np.zeros((abi.NLEVGRND, 2))
    fr[:4, 0] = [0.4, 0.3, 0.2, 0.1]
    fr[:4, 1] = [0.25, 0.25, 0.25, 0.25]
    A["rootfr"] = fr
    for (n, kind, t, u) in abi.ROOTMOIST_FIELDS:
        if n not in A or A[n].shape[-1] != abi.field_shape(kind, 1, 2, 1)[-1]:
            A[n] = np.zeros(abi.field_shape(kind, 1, 2, 1), dtype=np.dtype(t))
    A["rootfr"][:] = fr
    A["patch_column"][:] = 1
    A["itype"][:] = 1
    dz = A["dz"]
    dz[1 - LS:, 0] = 0.1
    A["watsat"][:, 0] = 0.4
    A["sucsat"][:, 0] = 100.0
    A["bsw"][:, 0] = 8.0
    A["t_soisno"][:, 0] = 285.0
    A["h2osoi_ice"][:, 0] = 0.0
    # level 1: s = 0.4 -> smp = -100*0.4^-8, between smpsc and smpso
    A["h2osoi_liq"][1 - LS, 0] = 0.16 * 0.1 * 1000.0
    # level 2: no liquid
    A["h2osoi_liq"][2 - LS, 0] = 0.0
    # level 3: liquid but T = tfrz - 2
    A["h2osoi_liq"][3 - LS, 0] = 0.3 * 0.1 * 1000.0
    A["t_soisno"][3 - LS, 0] = canopy_inputs.TFRZ - 2.0
    # level 4: half the pores iced, liquid fills the rest (s = 1)
    A["h2osoi_ice"][4 - LS, 0] = 0.2 * 0.1 * 917.0
    A["h2osoi_liq"][4 - LS, 0] = 0.3 * 0.1 * 1000.0
    A["rresis"][:] = -1.0
    b = abi.Bounds(1, 1, 1, 2)
    fp = np.array([1, 2], dtype=np.int32)
    io = abi.make_io(abi.RootMoistIO, abi.ROOTMOIST_FIELDS, A, 1, 2)
    assert L.oracle_root_moist_stress(C.byref(b), 2, _p(fp, C.c_int32), C.byref(io)) == 0
    smpso, smpsc = -74000.0, -275000.0
    r1 = (-100.0 * 0.4 ** -8 - smpsc) / (smpso - smpsc)
    r4 = min((0.2 / 0.4) * (-100.0 - smpsc) / (smpso - smpsc), 1.0)
    assert 0.0 < r1 < 1.0 and 0.0 < r4 < 1.0
    np.testing.assert_allclose(A["eff_porosity"][:4, 0], [0.4, 0.4, 0.4, 0.2], rtol=1e-15)
    np.testing.assert_allclose(A["h2osoi_liqvol"][:4, 0], [0.16, 0.0, 0.3, 0.2], rtol=1e-15)
    for p in range(2):
        bt = fr[0, p] * r1 + fr[3, p] * r4
        np.testing.assert_allclose(A["btran"][p], bt, rtol=1e-14)
        np.testing.assert_allclose(A["rootr"][:4, p], [fr[0, p] * r1 / bt, 0, 0, fr[3, p] * r4 / bt], rtol=1e-14)
        np.testing.assert_allclose(A["rresis"][[0, 3], p], [r1, r4], rtol=1e-14)
        assert (A["rresis"][[1, 2], p] == -1.0).all()       # not evaluated on dry / cold levels
    assert (A["rootr"][abi.NLEVSOI:] == 0.0).all()
