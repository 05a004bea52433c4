"""Restart files (ctsm_gb300/restart.py): the variables carry the reference's
restart names, types and dimensions (pinned from its restartvar declarations
into tests/golden/restart_vars.json by tests/golden/make_golden.py), and a
checkpoint survives checkpoint -> restart file -> checkpoint bit for bit."""
import json
import os

import numpy as np
import pytest

from ctsm_gb300 import abi, restart

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "restart_vars.json")
XTYPE = {"d": "ncd_double", "i": "ncd_int"}
DIM_KIND = {("column",): "C", ("pft",): "P", ("column", "levtot"): "SS"}


def _manifest_kinds():
    kinds = {}
    for table in (abi.SOILWATER_FIELDS, abi.SOILTEMP_FIELDS, abi.CANOPY_FIELDS, abi.SOILFLUXES_FIELDS,
                  abi.ROOTMOIST_FIELDS, abi.BAREGRND_FIELDS, abi.HYDROLOGY_FIELDS, abi.SOILRESIS_FIELDS,
                  abi.ROOTSINK_FIELDS):
        for f in table:
            kinds.setdefault(f[0], set()).add((f[1], f[2]))
    return kinds


def test_restart_variables_follow_the_reference_declarations():
    ref = json.load(open(GOLDEN))["vars"]
    kinds = _manifest_kinds()
    for var, (comp, code, dims) in restart.RESTART_VARS.items():
        r = ref[var]
        assert XTYPE[code] == r["xtype"], var
        # on file (C order): with switchdim the declared (dim1, dim2) are
        # stored as Fortran (dim2, dim1), i.e. (dim1, dim2) in C order
        want = (r["dim1name"],) if r["dim2name"] is None else \
            ((r["dim1name"], r["dim2name"]) if r["switchdim"] else (r["dim2name"], r["dim1name"]))
        assert dims == want, var
        kind, dt = next(iter(kinds[comp]))
        assert len(kinds[comp]) == 1 and kind == DIM_KIND[dims], (var, kinds[comp])
        assert dt == ("f8" if code == "d" else "i4"), var


def _synthetic(ncol=37, npatch=53, ngrid=3, seed=4):
    r = np.random.default_rng(seed)
    ck = restart.Checkpoint(ncol, npatch, ngrid)
    for var, (comp, code, dims) in restart.RESTART_VARS.items():
        kind = DIM_KIND[dims]
        shape = ck.shape(kind)
        a = r.integers(-12, 1, size=shape).astype(np.int32) if code == "i" else r.standard_normal(shape) * 300.0
        ck.fields[comp] = (kind, a)
    ck.fields["watsat"] = ("G", r.random(ck.shape("G")))          # a component without a restart variable
    ck.fields["forc_pbot"] = ("GR", r.random(ck.shape("GR")))
    return ck


def test_checkpoint_file_round_trip(tmp_path):
    ck = _synthetic()
    p = tmp_path / "state.ckpt"
    restart.write_checkpoint(p, ck)
    back = restart.read_checkpoint(p)
    assert (back.ncol, back.npatch, back.ngrid) == (ck.ncol, ck.npatch, ck.ngrid)
    assert list(back.fields) == list(ck.fields)
    for k, (kind, a) in ck.fields.items():
        assert back.fields[k][0] == kind and back.fields[k][1].dtype == a.dtype
        assert np.array_equal(back.fields[k][1], a)


def test_restart_file_layout_and_round_trip(tmp_path):
    pytest.importorskip("scipy")
    from scipy.io import netcdf_file
    ck = _synthetic()
    nc = tmp_path / "restart.nc"
    written = restart.checkpoint_to_restart(ck, nc)
    assert sorted(written) == sorted(restart.RESTART_VARS)
    f = netcdf_file(str(nc), "r", mmap=False)
    assert f.dimensions["column"] == ck.ncol and f.dimensions["pft"] == ck.npatch
    assert f.dimensions["levtot"] == abi.NLEVSNO + abi.NLEVGRND
    t = np.array(f.variables["T_SOISNO"][:])
    assert t.shape == (ck.ncol, abi.NLEVSNO + abi.NLEVGRND)
    # column c, level j (lower bound -nlevsno+1) of the level-major component
    assert t[5, 3] == ck.fields["t_soisno"][1][3, 5]
    assert np.array(f.variables["SNLSNO"][:]).dtype.kind == "i"
    f.close()
    template = restart.Checkpoint(ck.ncol, ck.npatch, ck.ngrid,
                                  {k: (kind, np.zeros_like(a)) for k, (kind, a) in ck.fields.items()})
    got, read = restart.restart_into_checkpoint(nc, template)
    assert sorted(read) == sorted(restart.RESTART_VARS)
    for k, (kind, a) in ck.fields.items():
        if k in ("watsat", "forc_pbot"):
            assert not got.fields[k][1].any()                   # not in the restart: the template's values
        else:
            assert got.fields[k][1].dtype == a.dtype and np.array_equal(got.fields[k][1], a), k


def test_restart_size_mismatch_is_refused(tmp_path):
    pytest.importorskip("scipy")
    ck = _synthetic()
    nc = tmp_path / "restart.nc"
    restart.checkpoint_to_restart(ck, nc)
    other = _synthetic(ncol=36)
    with pytest.raises(ValueError):
        restart.restart_into_checkpoint(nc, other)
