"""Root moisture stress (CanopyFluxesMod.F90:833-895 -> SoilMoistStressMod.F90)
on the GPU against the oracle: a full state with snow and frozen soil, plus
planted columns whose levels are dry (no liquid), cold (T <= tfrz - 2) or all
frozen (btran = 0, rootr = 0), over a patch filter with gaps."""
import copy
import ctypes as C

import numpy as np
import pytest

from ctsm_gb300 import abi, canopy, canopy_inputs, full_inputs as fi
from tests.parity import compare

pytestmark = pytest.mark.gpu
LS = -abi.NLEVSNO + 1
OUT = [n for (n, k, t, u) in abi.ROOTMOIST_FIELDS if u != "in"]


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def planted_state(ncol, seed):
    A, npatch, ngrid, rootr = fi.full_state(ncol, seed=seed)
    r = np.random.Generator(np.random.Philox(seed + 1))
    fi.add_rootmoist_fields(A, npatch, rootr, rng=r)
    A["rresis"][:] = -7.0                     # untouched where the stress is not evaluated
    soil = slice(1 - LS, abi.NLEVGRND + 1 - LS)
    dry, cold, frozen = (r.choice(ncol, 50, replace=False) for _ in range(3))
    for c in dry:
        js = r.choice(abi.NLEVSOI, 5, replace=False) + 1 - LS
        A["h2osoi_liq"][js, c] = 0.0
    for c in cold:
        js = r.choice(abi.NLEVSOI, 5, replace=False) + 1 - LS
        A["t_soisno"][js, c] = canopy_inputs.TFRZ - 2.0 - r.uniform(0.0, 1.0, 5)
        A["t_soisno"][js[0], c] = canopy_inputs.TFRZ - 2.0     # the boundary itself is stressed out
    A["t_soisno"][soil, frozen] = canopy_inputs.TFRZ - 5.0
    # ice-filled levels: the effective porosity reaches zero
    for c in r.choice(ncol, 50, replace=False):
        j = 1 - LS + int(r.integers(0, 3))
        A["h2osoi_ice"][j, c] = 2.0 * A["watsat"][j - (1 - LS), c] * A["dz"][j, c] * 917.0
    fp = np.sort(r.choice(np.arange(1, npatch + 1, dtype=np.int32), int(0.9 * npatch), replace=False))
    return A, npatch, fp.astype(np.int32), frozen


def test_root_moist_stress_matches_oracle(gpu_lib):
    from oracle import oracle as orc
    L = orc.lib()
    ncol = 4000
    A, npatch, fp, frozen = planted_state(ncol, seed=91)
    b = abi.Bounds(1, ncol, 1, npatch)
    canopy.set_params(canopy_inputs.make_params(), canopy_inputs.make_pftcon())
    L.oracle_set_canopy_params(C.byref(canopy_inputs.make_params()), C.byref(canopy_inputs.make_pftcon()), 1, 40)
    G, R = copy.deepcopy(A), copy.deepcopy(A)
    canopy.RootMoistStress(b, len(fp), fp, G)
    io = abi.make_io(abi.RootMoistIO, abi.ROOTMOIST_FIELDS, R, ncol, npatch)
    assert L.oracle_root_moist_stress(C.byref(b), len(fp), _p(fp, C.c_int32), C.byref(io)) == 0
    # columns without a filtered patch keep their porosity arrays
    cols = np.unique(A["patch_column"][fp - 1] - 1)
    errs, bad = compare({k: G[k][:, cols] if G[k].ndim == 2 and k in ("eff_porosity", "h2osoi_liqvol") else G[k]
                         for k in OUT},
                        {k: R[k][:, cols] if R[k].ndim == 2 and k in ("eff_porosity", "h2osoi_liqvol") else R[k]
                         for k in OUT}, OUT, 1e-12, {})
    assert not bad, {k: errs[k] for k in bad}
    # filtered patches of all-frozen columns: btran 0, rootr 0
    pcol = A["patch_column"][fp - 1] - 1
    fz = fp[np.isin(pcol, frozen)] - 1
    assert len(fz) > 0 and (G["btran"][fz] == 0.0).all() and (G["rootr"][:, fz] == 0.0).all()
    # where btran > 0 the normalised rootr sums to one; rresis in [0, 1] where evaluated
    live = fp[G["btran"][fp - 1] > 0] - 1
    assert np.abs(G["rootr"][:, live].sum(axis=0) - 1.0).max() < 1e-12
    ev = G["rresis"][:, fp - 1]
    assert ((ev == -7.0) | ((ev >= 0.0) & (ev <= 1.0))).all() and (ev != -7.0).any()
    # patches outside the filter are untouched
    out = np.setdiff1d(np.arange(npatch), fp - 1)
    assert (G["rresis"][:, out] == -7.0).all() and (G["btran"][out] == A["btran"][out]).all()
