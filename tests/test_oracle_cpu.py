"""CPU tests of the oracle: its solvers against scipy's LAPACK, its layer
structure and balance-check constants against the reference's own pins
(tests/golden/), and basic properties of its soil step."""
import copy
import ctypes as C
import json
import os

import numpy as np
import pytest

from ctsm_gb300 import abi, inputs
from oracle import oracle as orc

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DT = 1800.0


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


@pytest.mark.parametrize("seed,pivot", [(0, False), (1, False), (2, True), (3, True)])
def test_dgbsv_matches_lapack(seed, pivot):
    scipy_lapack = pytest.importorskip("scipy.linalg.lapack")
    r = np.random.default_rng(seed)
    n, kl, ku = 38, 2, 2
    A = np.zeros((n, n))
    for i in range(n):
        for j in range(max(0, i - kl), min(n, i + ku + 1)):
            A[i, j] = r.normal()
        if not pivot:
            A[i, i] = 10.0 + abs(A[i]).sum()
    b = r.normal(size=n)
    ldab = 2 * kl + ku + 1
    ab = np.zeros((ldab, n))               # LAPACK band storage, rows kl.. used
    for j in range(n):
        for i in range(max(0, j - ku), min(n, j + kl + 1)):
            ab[kl + ku + i - j, j] = A[i, j]
    ab_f = np.asfortranarray(ab.copy())
    x = b.copy()
    ipiv = np.zeros(n, dtype=np.int32)
    info = orc.lib().oracle_dgbsv(n, kl, ku, _p(ab_f), ldab, _p(ipiv, C.c_int), _p(x))
    assert info == 0
    lub, piv, xs, info2 = scipy_lapack.dgbsv(kl, ku, ab.copy(), b.copy())
    assert info2 == 0
    np.testing.assert_allclose(x, xs, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(A @ x, b, rtol=1e-10, atol=1e-10)
    if pivot:
        assert (ipiv != np.arange(1, n + 1)).any()


def test_dgbsv_reports_singular():
    n, kl, ku = 6, 2, 2
    ab = np.zeros((2 * kl + ku + 1, n), order="F")
    ab[kl + ku, :] = 1.0
    ab[kl + ku, 3] = 0.0          # zero column 4 -> info = 4
    x = np.ones(n)
    ipiv = np.zeros(n, dtype=np.int32)
    info = orc.lib().oracle_dgbsv(n, kl, ku, _p(ab), 2 * kl + ku + 1, _p(ipiv, C.c_int), _p(x))
    assert info == 4


def test_tridiagonal_matches_lapack():
    scipy_lapack = pytest.importorskip("scipy.linalg.lapack")
    r = np.random.default_rng(7)
    n = 21
    a, c = r.normal(size=n), r.normal(size=n)
    b = 5.0 + np.abs(a) + np.abs(c)
    rhs = r.normal(size=n)
    u = np.zeros(n)
    orc.lib().oracle_tridiagonal(n, _p(a), _p(b), _p(c), _p(rhs), _p(u))
    _, _, _, xs, info = scipy_lapack.dgtsv(a[1:].copy(), b.copy(), c[:-1].copy(), rhs.copy())
    assert info == 0
    np.testing.assert_allclose(u, xs, rtol=1e-12)


def test_layer_structure_matches_tech_note_table():
    g = json.load(open(os.path.join(GOLD, "layer_table_20sl.json")))
    dz, z, zi = inputs.layer_structure_20sl()
    for (lev, zt, dzt, zht) in g["rows"]:
        assert round(z[lev - 1], 3) == pytest.approx(zt, abs=1.01e-3)
        assert round(dz[lev - 1], 3) == pytest.approx(dzt, abs=1.01e-3)
        assert round(zi[lev], 3) == pytest.approx(zht, abs=1.01e-3)


def test_skip_steps_golden():
    """skip_steps = max(2, nint(3600/dtime)) + 1 (BalanceCheckMod.F90:91)."""
    from ctsm_gb300 import balance
    g = json.load(open(os.path.join(GOLD, "skip_steps.json")))
    for dtime, n in g["cases"]:
        assert balance.skip_steps(float(dtime)) == n


def _oracle_step(A, npatch, which=("water", "temp")):
    L = orc.lib()
    ncol = A["zwt"].shape[0]
    b = abi.Bounds(1, ncol, 1, npatch)
    f = np.arange(1, ncol + 1, dtype=np.int32)
    if "water" in which:
        io = abi.make_io(abi.SoilWaterIO, abi.SOILWATER_FIELDS, A, ncol)
        assert L.oracle_soilwater(C.byref(b), ncol, _p(f, C.c_int32), C.byref(io), 6.0, DT) == 0
    if "temp" in which:
        io = abi.make_io(abi.SoilTempIO, abi.SOILTEMP_FIELDS, A, ncol, npatch)
        assert L.oracle_soiltemperature(C.byref(b), ncol, _p(f, C.c_int32), C.byref(io), DT, 0) == 0


def test_oracle_deterministic_and_thread_invariant():
    A, npatch = inputs.soil_columns(777, seed=9, snow=True, nbedrock=(3, 20), forcing="full", npatch_max=3)
    B, C2 = copy.deepcopy(A), copy.deepcopy(A)
    _oracle_step(B, npatch)
    _oracle_step(C2, npatch)
    for k in ("h2osoi_liq", "t_soisno", "qcharge", "xmf"):
        np.testing.assert_array_equal(B[k], C2[k])


def test_zd09_water_conservation():
    """ZD09 conserves water: the tridiagonal fluxes telescope, so the change of
    column liquid equals (infiltration - root sink - aquifer recharge) * dtime
    (recharge counted only when the water table is below the column)."""
    A, npatch = inputs.soil_columns(2000, seed=4, zwt=(0.5, 12.0))
    LS = -abi.NLEVSNO + 1
    w0 = A["h2osoi_liq"][1 - LS:abi.NLEVSOI + 1 - LS].sum(axis=0)
    R = copy.deepcopy(A)
    _oracle_step(R, npatch, which=("water",))
    w1 = R["h2osoi_liq"][1 - LS:abi.NLEVSOI + 1 - LS].sum(axis=0)
    deep = A["zwt"] > A["zi"][abi.NLEVSOI + abi.NLEVSNO]
    net = (A["qflx_infl"] - A["qflx_rootsoi"].sum(axis=0) - np.where(deep, R["qcharge"], 0.0)) * DT
    err = (w1 - w0) - net
    assert np.abs(err).max() < 1e-9       # the reference's h2o warning threshold (mm)


def test_libm_noise_moves_results_and_resets():
    A, npatch = inputs.soil_columns(64, seed=2)
    L = orc.lib()
    B = copy.deepcopy(A)
    _oracle_step(B, npatch)
    L.oracle_set_libm_noise(4, 1)
    try:
        N = copy.deepcopy(A)
        _oracle_step(N, npatch)
    finally:
        L.oracle_set_libm_noise(0, 0)
    assert np.abs(N["smp_l"] - B["smp_l"]).max() > 0
    assert np.abs(N["h2osoi_liq"] - B["h2osoi_liq"]).max() / np.abs(B["h2osoi_liq"]).max() < 1e-12
    Z = copy.deepcopy(A)
    _oracle_step(Z, npatch)
    np.testing.assert_array_equal(Z["smp_l"], B["smp_l"])
