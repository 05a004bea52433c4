"""CPU tests of the canopy oracle: quadratic against the reference's own
unit test (src/utils/test/quadratic_test/test_quadratic.pf), QSat against its
coefficient table, and properties of CanopyFluxes."""
import copy
import ctypes as C
import json
import os

import numpy as np
import pytest

from ctsm_gb300 import abi, canopy_inputs as ci
from oracle import oracle as orc

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
EPS = np.finfo(np.float64).eps


def quad(a, b, c):
    r1, r2 = C.c_double(), C.c_double()
    rc = orc.lib().oracle_quadratic(a, b, c, C.byref(r1), C.byref(r2))
    return rc, r1.value, r2.value


def test_quadratic_known_answers():
    g = json.load(open(os.path.join(GOLD, "quadratic_kat.json")))
    tol, tol_big = g["tol"], g["tol_big"]
    zr = g["zero_root"]
    for a in zr["a"]:
        rc, r1, r2 = quad(a, zr["b"], zr["c"])
        assert rc == 0 and abs(r1 - zr["r1"]) <= tol and abs(r2 - zr["r2"]) <= tol
    sr = g["simple_roots"]
    for a, b, c, e1, e2 in zip(sr["a"], sr["b"], sr["c"], sr["r1"], sr["r2"]):
        rc, r1, r2 = quad(a, b, c)
        assert rc == 0 and abs(r1 - e1) <= tol and abs(r2 - e2) <= tol
        for r in (r1, r2):
            assert abs(a * r * r + b * r + c) <= tol
    nz = g["near_zero_sqrts"]
    for pe in nz["pert_eps"]:
        rc, r1, r2 = quad(nz["a"], nz["b"], nz["c"] + pe * EPS)
        assert rc == 0 and abs(r1 - nz["r1"]) <= tol_big and abs(r1 - r2) <= tol_big
    for e in g["errors"]:
        c = e["c"] if "c" in e else e["b"] ** 2 / 4 + e["c_plus_eps"] * EPS
        rc, _, _ = quad(e["a"], e["b"], c)
        assert rc == 5     # CTSMG_E_DISCRIMINANT: the reference's endrun


def test_qsat_polynomials_match_coefficient_table():
    g = json.load(open(os.path.join(GOLD, "qsat_coeffs.json")))["coeffs"]
    L = orc.lib()
    for T in (200.0, 250.0, 273.149, 273.15, 290.0, 320.0, 400.0):
        qs, es, qd = C.c_double(), C.c_double(), C.c_double()
        L.oracle_qsat(T, 101325.0, C.byref(qs), C.byref(es), C.byref(qd))
        td = min(100.0, max(-75.0, T - 273.15))
        co, cd = (g["a"], g["b"]) if td >= 0 else (g["c"], g["d"])
        def horner(cs):
            v = cs[8]
            for k in range(7, -1, -1):
                v = cs[k] + td * v
            return v
        ref = horner(co) * 100.0
        assert es.value == pytest.approx(ref, rel=1e-15)
        refd = horner(cd) * 100.0
        vp = 1.0 / (101325.0 - 0.378 * ref)
        assert qs.value == pytest.approx(ref * 0.622 * vp, rel=1e-13)
        assert qd.value == pytest.approx(refd * 0.622 * vp * vp * 101325.0, rel=1e-12)


def _run(A, npatch, ncol, ngrid, itmax=40, method=1):
    L = orc.lib()
    L.oracle_set_canopy_params(C.byref(ci.make_params()), C.byref(ci.make_pftcon()), method, itmax)
    b = abi.Bounds(1, ncol, 1, npatch)
    io = abi.make_io(abi.CanopyIO, abi.CANOPY_FIELDS, A, ncol, npatch, ngrid, 1)
    f = np.arange(1, npatch + 1, dtype=np.int32)
    e = C.c_int(0)
    return L.oracle_canopyfluxes(C.byref(b), npatch, f.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(io), 1800.0,
                                 C.byref(e))


def test_canopy_oracle_properties():
    A, npatch, ncol, ngrid = ci.canopy_patches(5000, seed=5)
    assert _run(A, npatch, ncol, ngrid) == 0
    assert np.abs(A["err_canopy"]).max() < 1e-9          # leaf energy balance closes
    it = A["num_iter"]
    assert it.min() >= 3 and it.max() <= 41               # itmin = 2, up to itmax + 1 passes
    assert (A["rssun"] > 0).all() and (A["rssun"] <= 2.0e4 + 1e-9).all()
    night = A["parsun_z"] <= 0
    assert (A["psnsun"][night] == 0).all()
    assert np.isfinite(A["t_veg"]).all()


def test_canopy_itmax_caps_passes():
    A, npatch, ncol, ngrid = ci.canopy_patches(2000, seed=6)
    assert _run(A, npatch, ncol, ngrid, itmax=3) == 0
    assert A["num_iter"].max() <= 4


def test_ball_berry_option_runs():
    A, npatch, ncol, ngrid = ci.canopy_patches(1000, seed=7)
    assert _run(A, npatch, ncol, ngrid, method=0) == 0
    assert np.abs(A["err_canopy"]).max() < 1e-9
