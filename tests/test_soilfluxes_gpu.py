"""SoilFluxes drop-in (SoilFluxesMod.F90) against the oracle, on a state
stepped by the oracle through CanopyFluxes, the root sink and SoilTemperature
(the temperatures before SoilTemperature saved as tssbef / t_h2osfc_bef).
Some columns get a nearly empty top layer so that both evaporation limits
(:282-297 snow, :317-327 top-soil ice) act."""
import copy
import ctypes as C

import numpy as np
import pytest

from ctsm_gb300 import abi, canopy_inputs, full_inputs as fi, soil
from tests.parity import compare

pytestmark = pytest.mark.gpu
DT = 1800.0
LS = -abi.NLEVSNO + 1
OUT = [n for (n, k, t, u) in abi.SOILFLUXES_FIELDS if u != "in"]


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def stepped_state(ncol, seed):
    from oracle import oracle as orc
    L = orc.lib()
    A, npatch, ngrid, rootr = fi.full_state(ncol, seed=seed)
    for (n, kind, t, u) in abi.SOILFLUXES_FIELDS:
        if n not in A:
            A[n] = np.zeros(abi.field_shape(kind, ncol, npatch, ngrid), dtype=np.dtype(t))
    b = abi.Bounds(1, ncol, 1, npatch)
    fc = np.arange(1, ncol + 1, dtype=np.int32)
    fp = np.arange(1, npatch + 1, dtype=np.int32)
    L.oracle_set_canopy_params(C.byref(canopy_inputs.make_params()), C.byref(canopy_inputs.make_pftcon()), 1, 40)
    A["cgrnds"][:] = 0.0
    A["cgrndl"][:] = 0.0
    ci = abi.make_io(abi.CanopyIO, abi.CANOPY_FIELDS, A, ncol, npatch, ngrid, 1)
    e = C.c_int(0)
    assert L.oracle_canopyfluxes(C.byref(b), npatch, _p(fp, C.c_int32), C.byref(ci), DT, C.byref(e)) == 0
    L.oracle_rootsink(ncol, npatch, _p(A["col_patchi"], C.c_int32), _p(A["col_npatches"], C.c_int32),
                      _p(A["wtcol"]), _p(A["qflx_tran_veg"]), _p(np.ascontiguousarray(rootr)), _p(A["qflx_rootsoi"]))
    A["tssbef"][:] = A["t_soisno"]
    A["t_h2osfc_bef"][:] = A["t_h2osfc"]
    st = abi.make_io(abi.SoilTempIO, abi.SOILTEMP_FIELDS, A, ncol, npatch)
    assert L.oracle_soiltemperature(C.byref(b), ncol, _p(fc, C.c_int32), C.byref(st), DT, 0) == 0
    return A, npatch, b, fc, fp


def test_soilfluxes_matches_oracle(gpu_lib):
    from oracle import oracle as orc
    L = orc.lib()
    A, npatch, b, fc, fp = stepped_state(3000, seed=81)
    ncol = A["zwt"].shape[0]
    r = np.random.Generator(np.random.Philox(82))
    snow = np.nonzero(A["snl"] < 0)[0]
    bare = np.nonzero(A["snl"] == 0)[0]
    tiny_snow = r.choice(snow, 40, replace=False)
    tiny_ice = r.choice(bare, 40, replace=False)
    for c in tiny_snow:
        j = A["snl"][c] + 1 - LS
        A["h2osoi_ice"][j, c], A["h2osoi_liq"][j, c] = 1e-4, 1e-5
    A["h2osoi_ice"][1 - LS, tiny_ice] = 1e-3
    A["h2osoi_liq"][1 - LS, tiny_ice] = 1e-3
    pcol = A["patch_column"] - 1
    for c in tiny_ice:                      # evaporating, so the top-soil ice limit is reached
        A["qflx_ev_snow"][pcol == c] = 1e-5
    G, R = copy.deepcopy(A), copy.deepcopy(A)
    soil.SoilFluxes(b, ncol, fc, npatch, fp, G, DT)
    io = abi.make_io(abi.SoilFluxesIO, abi.SOILFLUXES_FIELDS, R, ncol, npatch)
    assert L.oracle_soilfluxes(C.byref(b), ncol, _p(fc, C.c_int32), npatch, _p(fp, C.c_int32), C.byref(io), DT) == 0
    # both limits acted on some patches
    snow_limited = np.isin(pcol, tiny_snow) & (R["qflx_ev_snow"] < A["qflx_ev_snow"] - 1e-12)
    ice_limited = np.isin(pcol, tiny_ice) & (R["qflx_solidevap_from_top_layer"] > 0) & \
        np.isclose(R["qflx_solidevap_from_top_layer"], 1e-3 / DT)
    assert snow_limited.sum() > 5 and ice_limited.sum() > 5, (snow_limited.sum(), ice_limited.sum())
    resid = ("errsoi_patch", "errsoi_col")
    errs, bad = compare(G, R, [k for k in OUT if k not in resid], 1e-9, {})
    assert not bad, {k: errs[k] for k in bad}
    # errsoi is a residual of fluxes of hundreds of W/m2: compared absolutely
    for k in resid:
        assert np.abs(G[k] - R[k]).max() < 1e-9, (k, np.abs(G[k] - R[k]).max())
    # SoilTemperature conserves energy: the reference's errsoi warning threshold
    assert np.abs(R["errsoi_col"]).max() < 1e-5 and np.abs(G["errsoi_col"]).max() < 1e-5
