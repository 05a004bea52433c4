"""The oracle's drainage routines close the column water budget
(SoilHydrologyMod.F90:1645-1929, 2029-2565): SubsurfaceLateralFlow changes
liquid + ice + h2osfc by -(qflx_drain + qflx_ice_runoff_xs) dtime and
PerchedLateralFlow liquid by -qflx_drain_perched dtime."""
import ctypes as C

import numpy as np

from ctsm_gb300 import abi, inputs, full_inputs as fi

LS = -abi.NLEVSNO + 1
DT = 1800.0


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def _state(seed):
    A, _ = inputs.soil_columns(800, seed=seed, snow=True, nbedrock=(3, 20), zwt=(0.2, 9.0))
    fi.add_hydrology_fields(A, np.random.Generator(np.random.Philox(seed)))
    return A


def _run(A, which):
    from oracle import oracle as orc
    ncol = A["zwt"].shape[0]
    io = abi.make_io(abi.HydrologyIO, abi.HYDROLOGY_FIELDS, A, ncol)
    f = np.arange(1, ncol + 1, dtype=np.int32)
    P = abi.SoilHydrologyParams(0.01, 1.0, 1.0e-2, 1.0e-5, 6.0, 0.5, 0.4, 0.13, 1)
    assert orc.lib().oracle_hydrology(C.byref(abi.Bounds(1, ncol, 1, 1)), ncol, _p(f, C.c_int32), C.byref(io),
                                      which, C.byref(P), DT) == 0


def test_drainage_closes_column_water():
    A = _state(51)
    _run(A, 1)                         # PerchedWaterTable sets the frost table
    soil = slice(1 - LS, abi.NLEVSOI + 1 - LS)
    w0 = A["h2osoi_liq"][soil].sum(0)
    _run(A, 3)
    assert (A["qflx_drain_perched"] > 0).any()
    np.testing.assert_allclose(A["h2osoi_liq"][soil].sum(0) - w0, -A["qflx_drain_perched"] * DT, atol=1e-9)
    w0 = A["h2osoi_liq"][soil].sum(0) + A["h2osoi_ice"][soil].sum(0) + A["h2osfc"]
    _run(A, 4)
    w1 = A["h2osoi_liq"][soil].sum(0) + A["h2osoi_ice"][soil].sum(0) + A["h2osfc"]
    assert (A["qflx_latflow_out"] > 0).any() and (A["qflx_latflow_out"] == 0).any()
    np.testing.assert_allclose(w1 - w0, -(A["qflx_drain"] + A["qflx_ice_runoff_xs"]) * DT, atol=1e-8)
    assert (A["zwt"] >= 0).all() and (A["zwt"] <= 80).all()
