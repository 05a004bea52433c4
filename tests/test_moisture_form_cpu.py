"""The oracle's moisture form on the CPU: its dgtsv restatement against
scipy's LAPACK dgtsv, water conservation with the zero-flux bottom boundary,
and the C-ABI's namelist consistency checks (SoilWaterMovementMod.F90:190-197)."""
import ctypes as C

import numpy as np
import pytest

from ctsm_gb300 import abi, inputs

LS = -abi.NLEVSNO + 1


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


@pytest.mark.parametrize("n,seed,dominant", [(3, 0, True), (2, 1, False), (5, 2, False), (20, 3, True),
                                             (20, 4, False), (13, 5, False)])
def test_dgtsv_matches_lapack(n, seed, dominant):
    from oracle import oracle as orc
    lapack = pytest.importorskip("scipy.linalg.lapack")
    r = np.random.default_rng(seed)
    dl, du = r.uniform(-2, 2, n - 1), r.uniform(-2, 2, n - 1)
    d = r.uniform(-2, 2, n) + 5.0 if dominant else r.uniform(-0.1, 0.1, n)
    b = r.uniform(-1, 1, n)
    _, _, _, x_ref, info = lapack.dgtsv(dl.copy(), d.copy(), du.copy(), b.copy())
    a = [np.ascontiguousarray(v.copy()) for v in (dl if n > 1 else np.zeros(1), d, du if n > 1 else np.zeros(1), b)]
    got = orc.lib().oracle_dgtsv(n, *[_p(v) for v in a])
    assert got == info == 0
    np.testing.assert_allclose(a[3], x_ref, rtol=1e-13, atol=1e-15)
    if not dominant and n >= 5:       # partial pivoting really exchanged rows somewhere
        assert (np.abs(d[:-1]) < np.abs(dl)).any()


def test_dgtsv_zero_pivot():
    from oracle import oracle as orc
    dl, d, du, b = (np.array(v, float) for v in ([0.0], [0.0, 1.0], [1.0], [1.0, 1.0]))
    assert orc.lib().oracle_dgtsv(2, _p(dl), _p(d), _p(du), _p(b)) == 1


def test_zero_flux_conserves_water():
    """With bc_zero_flux every accepted sub-step moves (qflx_infl - sum of the
    root sink) * dtsub into the column, and the over-saturation pass only
    moves water upward: the column total changes by exactly that."""
    from oracle import oracle as orc
    L = orc.lib()
    ncol = 500
    A, _ = inputs.soil_columns(ncol, seed=41, snow=True, nbedrock=(3, 20), forcing="full")
    r = np.random.default_rng(42)
    A["qflx_rootsoi"][:] = r.uniform(0.0, 2e-5, A["qflx_rootsoi"].shape)
    w0 = A["h2osoi_liq"][1 - LS:abi.NLEVSOI + 1 - LS].copy()
    nml = abi.soilwater_movement_nml(1)
    io = abi.make_io(abi.SoilWaterIO, abi.SOILWATER_FIELDS + abi.SOILWATER_EXTRA, A, ncol)
    f = np.arange(1, ncol + 1, dtype=np.int32)
    e = C.c_int(0)
    assert L.oracle_soilwater_mf(C.byref(abi.Bounds(1, ncol, 1, 1)), ncol, _p(f, C.c_int32), C.byref(io), 6.0,
                                 1800.0, C.byref(nml), C.byref(e)) == 0
    mask = np.arange(1, abi.NLEVSOI + 1)[:, None] <= A["nbedrock"][None, :]
    dw = ((A["h2osoi_liq"][1 - LS:abi.NLEVSOI + 1 - LS] - w0) * mask).sum(0)
    expect = (A["qflx_infl"] - (A["qflx_rootsoi"] * mask).sum(0)) * 1800.0
    assert np.abs(dw - expect).max() < 1e-8
    assert (A["qcharge"] == 0.0).all() and (A["num_substeps"] >= 1).all()


def test_namelist_consistency_checks():
    from ctsm_gb300 import build
    from ctsm_gb300._lib import load
    build.build()
    L = load()
    nml = abi.soilwater_movement_nml
    assert L.ctsmg_set_soilwater_movement(C.byref(nml(1))) == 0
    assert L.ctsmg_set_soilwater_movement(C.byref(nml(1, lower=1, use_bedrock=0))) == 0
    assert L.ctsmg_set_soilwater_movement(C.byref(nml(1, lower=3, use_bedrock=0))) == 0
    assert L.ctsmg_set_soilwater_movement(C.byref(nml(0, use_bedrock=0))) == 0
    assert L.ctsmg_set_soilwater_movement(C.byref(nml(0, lower=2, use_bedrock=0))) == 1   # ZD09 needs bc_aquifer
    assert L.ctsmg_set_soilwater_movement(C.byref(nml(1, lower=1, use_bedrock=1))) == 1   # bedrock needs zero flux
    assert L.ctsmg_set_soilwater_movement(C.byref(nml(1, upper=0))) == 10                 # bc_head
    assert L.ctsmg_set_soilwater_movement(C.byref(nml(1, lower=4, use_bedrock=0))) == 10  # no aquifer case
    assert L.ctsmg_set_soilwater_movement(C.byref(nml(2))) == 10                          # mixed form is empty
    assert L.ctsmg_set_soilwater_movement(C.byref(nml(0, use_bedrock=0))) == 0
