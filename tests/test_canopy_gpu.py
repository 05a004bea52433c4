"""Parity of the CUDA CanopyFluxes + Photosynthesis drop-in call with the oracle."""
import copy
import ctypes as C

import numpy as np
import pytest

from ctsm_gb300 import abi, canopy_inputs as ci
from tests.parity import compare, noise_spread

pytestmark = pytest.mark.gpu
DT = 1800.0
OUT = [n for (n, k, t, u) in abi.CANOPY_FIELDS if u != "in"]


def run_oracle(A, npatch, ncol, ngrid, filt, method=1, itmax=40):
    from oracle import oracle as orc
    L = orc.lib()
    L.oracle_set_canopy_params(C.byref(ci.make_params()), C.byref(ci.make_pftcon()), method, itmax)
    b = abi.Bounds(1, ncol, 1, npatch)
    io = abi.make_io(abi.CanopyIO, abi.CANOPY_FIELDS, A, ncol, npatch, ngrid, 1)
    f = np.ascontiguousarray(filt, np.int32)
    e = C.c_int(0)
    rc = L.oracle_canopyfluxes(C.byref(b), len(f), f.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(io), DT,
                               C.byref(e))
    assert rc == 0, (rc, e.value)


@pytest.fixture(scope="module")
def canopy_lib(gpu_lib):
    from ctsm_gb300 import canopy
    canopy.set_params()
    return canopy


def _case(canopy_lib, npatch, seed, **kw):
    A, npatch, ncol, ngrid = ci.canopy_patches(npatch, seed=seed, **kw)
    filt = np.arange(1, npatch + 1, dtype=np.int32)
    G, R = copy.deepcopy(A), copy.deepcopy(A)
    run_oracle(R, npatch, ncol, ngrid, filt)
    canopy_lib.CanopyFluxes(abi.Bounds(1, ncol, 1, npatch), npatch, filt, G, DT, ngrid)
    return A, G, R, npatch, ncol, ngrid, filt


# Outputs that are differences of nearly equal operands: the canopy water
# stores after evaporation (liqcan/snocan = max(0, store + (tran - evap) dtime),
# CanopyFluxesMod.F90:1640-1652) and the ground sensible heat, whose driving
# temperature difference wtal*t_grnd - wtl0*t_veg - wta0*thm is a difference of
# ~300 K operands (:1493-1503).  They are judged against the oracle's own
# spread under libm noise plus a +-4 ulp perturbation of every input.
CANOPY_CANCELLATION = ("liqcan", "snocan", "eflx_sh_grnd", "eflx_sh_snow", "eflx_sh_soil", "eflx_sh_h2osfc",
                       "qflx_evap_soi", "qflx_ev_snow", "qflx_ev_soil", "qflx_ev_h2osfc")


def _band(A, R, npatch, ncol, ngrid, filt):
    """Acceptance band of the cancellation outputs: the oracle's spread, plus
    for the canopy water stores 1e-9 of the incoming stores (the operands of
    store + (tran - evap) * dtime)."""
    sp = noise_spread(lambda B: run_oracle(B, npatch, ncol, ngrid, filt), A, R,
                      fields=CANOPY_CANCELLATION, input_ulps=4)
    operand = np.abs(A["liqcan"]) + np.abs(A["snocan"])
    sp["liqcan"] = sp["liqcan"] + 1e-9 * operand
    sp["snocan"] = sp["snocan"] + 1e-9 * operand
    return sp


def test_canopy_matches_oracle(canopy_lib):
    A, G, R, npatch, ncol, ngrid, filt = _case(canopy_lib, 30000, seed=2)
    np.testing.assert_array_equal(G["num_iter"], R["num_iter"])
    spread = _band(A, R, npatch, ncol, ngrid, filt)
    # err_canopy is the leaf energy-balance residual (~1e-12 W/m2): it is
    # checked absolutely below, not relatively
    errs, bad = compare(G, R, [k for k in OUT if k != "err_canopy"], 1e-9, spread)
    assert not bad, {k: errs[k] for k in bad}
    assert np.abs(G["err_canopy"] - R["err_canopy"]).max() < 1e-9


def test_canopy_energy_balance_closes(canopy_lib):
    """The leaf energy balance the reference reports (CanopyFluxesMod.F90:1750-1765
    warns above 0.1 W/m2) closes to round-off on every patch."""
    A, G, R, *_ = _case(canopy_lib, 8000, seed=3)
    assert np.abs(G["err_canopy"]).max() < 1e-8


@pytest.mark.parametrize("npatch", [1, 33, 257])
def test_canopy_ragged(canopy_lib, npatch):
    A, G, R, npatch, ncol, ngrid, filt = _case(canopy_lib, npatch, seed=10 + npatch)
    np.testing.assert_array_equal(G["num_iter"], R["num_iter"])
    spread = _band(A, R, npatch, ncol, ngrid, filt)
    errs, bad = compare(G, R, [k for k in OUT if k != "err_canopy"], 1e-9, spread)
    assert not bad, {k: errs[k] for k in bad}


def test_canopy_ball_berry_matches_oracle(canopy_lib, gpu_lib):
    """Ball-Berry 1987 stomatal conductance (stomatalcond_method = 0,
    PhotosynthesisMod.F90:2684-2690 in ci_func, :1962-1974 for rs): the same
    parity bar as the Medlyn default, with identical pass counts."""
    gpu_lib.init(stomatalcond_method=0)
    try:
        A, npatch, ncol, ngrid = ci.canopy_patches(20000, seed=5)
        filt = np.arange(1, npatch + 1, dtype=np.int32)
        G, R = copy.deepcopy(A), copy.deepcopy(A)
        run_oracle(R, npatch, ncol, ngrid, filt, method=0)
        canopy_lib.CanopyFluxes(abi.Bounds(1, ncol, 1, npatch), npatch, filt, G, DT, ngrid)
        # the Medlyn default gives other conductances: the method did switch
        M = copy.deepcopy(A)
        run_oracle(M, npatch, ncol, ngrid, filt, method=1)
        assert np.abs(M["rssun"] - R["rssun"]).max() > 1.0
        np.testing.assert_array_equal(G["num_iter"], R["num_iter"])
        sp = noise_spread(lambda B: run_oracle(B, npatch, ncol, ngrid, filt, method=0), A, R,
                          fields=CANOPY_CANCELLATION, input_ulps=4)
        operand = np.abs(A["liqcan"]) + np.abs(A["snocan"])
        sp["liqcan"] = sp["liqcan"] + 1e-9 * operand
        sp["snocan"] = sp["snocan"] + 1e-9 * operand
        errs, bad = compare(G, R, [k for k in OUT if k != "err_canopy"], 1e-9, sp)
        assert not bad, {k: errs[k] for k in bad}
        assert np.abs(G["err_canopy"] - R["err_canopy"]).max() < 1e-9
    finally:
        gpu_lib.init()
