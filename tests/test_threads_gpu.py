"""The boundary's threading contract.  The reference makes its column calls
inside the !$OMP PARALLEL DO over clumps of src/main/clm_driver.F90:525, so a
drop-in is called from several host threads at once, each with its own clump
(disjoint bounds and filters) of the same derived-type arrays.  Here four
Python threads (ctypes releases the GIL for the call) run ctsmg_soilwater and
then ctsmg_soiltemperature on four clumps of one set of arrays at the same
time, each passing pointers into the shared arrays at its clump's first
column / patch with the full leading dimensions, as c_loc(inst%field(begc, lb))
does.  The results are bit-identical to the same calls made one after another,
and within 1e-9 of the oracle."""
import copy
import ctypes as C
import threading

import numpy as np
import pytest

from ctsm_gb300 import abi, inputs
from ctsm_gb300._lib import load, check
from tests.parity import compare, noise_spread, fgr_rounding_bound

pytestmark = pytest.mark.gpu
DT = 1800.0
NCLUMP = 4


def _clump_io(cls, fields, A, ncol, npatch, begc, begp):
    """io struct of one clump: each pointer at the clump's first column (or
    patch) of the shared arrays, leading dimensions of the whole arrays."""
    io = abi.make_io(cls, fields, A, ncol, npatch) if npatch is not None else abi.make_io(cls, fields, A, ncol)
    for (n, kind, t, _) in fields:
        off = (begp - 1) if kind in ("P", "PL", "PS", "PG") else (begc - 1)
        esize = 8 if t == abi.F64 else 4
        base = A[n].ctypes.data + off * esize
        setattr(io, n, C.cast(C.c_void_p(base), abi._ptr_type(t)))
    return io


def _clumps(A, ncol, npatch):
    per = ncol // NCLUMP
    out = []
    for k in range(NCLUMP):
        c0, c1 = k * per + 1, (k + 1) * per if k < NCLUMP - 1 else ncol
        p0 = int(A["col_patchi"][c0 - 1])
        p1 = int(A["col_patchi"][c1 - 1] + A["col_npatches"][c1 - 1] - 1)
        # the clump's filter: its columns in a scrambled order with a few left out
        r = np.random.Generator(np.random.Philox(90 + k))
        f = r.permutation(np.arange(c0, c1 + 1, dtype=np.int32))[: (c1 - c0 + 1) - 7]
        out.append((abi.Bounds(c0, c1, p0, p1), np.ascontiguousarray(f)))
    return out


def _call(L, A, ncol, npatch, bnd, filt):
    fp = filt.ctypes.data_as(C.POINTER(C.c_int32))
    sw = _clump_io(abi.SoilWaterIO, abi.SOILWATER_FIELDS, A, ncol, None, bnd.begc, bnd.begp)
    st = _clump_io(abi.SoilTempIO, abi.SOILTEMP_FIELDS, A, ncol, npatch, bnd.begc, bnd.begp)
    check(L.ctsmg_soilwater(C.byref(bnd), len(filt), fp, C.byref(sw), DT))
    check(L.ctsmg_soiltemperature(C.byref(bnd), len(filt), fp, C.byref(st), DT))


def test_concurrent_clumps_match_serial_and_oracle(gpu_lib):
    from oracle import oracle as orc
    L = load()
    ncol = 4 * 6000
    A, npatch = inputs.soil_columns(ncol, seed=71, snow=True, nbedrock=(3, 20), forcing="full", npatch_max=3,
                                    h2osfc=True)
    clumps = _clumps(A, ncol, npatch)
    # serial: one clump after the other
    S = copy.deepcopy(A)
    for bnd, f in clumps:
        _call(L, S, ncol, npatch, bnd, f)
    # concurrent: one host thread per clump, started together
    P = copy.deepcopy(A)
    errors = []
    go = threading.Barrier(NCLUMP)

    def worker(bnd, f):
        try:
            go.wait()
            for _ in range(1):
                _call(L, P, ncol, npatch, bnd, f)
        except Exception as e:                 # reported below
            errors.append(e)
    ts = [threading.Thread(target=worker, args=c) for c in clumps]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=300)
    assert not errors, errors
    assert not any(t.is_alive() for t in ts)
    for k in A:
        assert np.array_equal(P[k], S[k], equal_nan=True), k
    # oracle over the union of the clump filters (the clumps are independent)
    R = copy.deepcopy(A)
    filt = np.concatenate([f for _, f in clumps])
    b = abi.Bounds(1, ncol, 1, npatch)
    Lo = orc.lib()
    fp = filt.ctypes.data_as(C.POINTER(C.c_int32))

    def run(B):
        sw = abi.make_io(abi.SoilWaterIO, abi.SOILWATER_FIELDS, B, ncol)
        st = abi.make_io(abi.SoilTempIO, abi.SOILTEMP_FIELDS, B, ncol, npatch)
        assert Lo.oracle_soilwater(C.byref(b), len(filt), fp, C.byref(sw), 6.0, DT) == 0
        assert Lo.oracle_soiltemperature(C.byref(b), len(filt), fp, C.byref(st), DT, 0) == 0
    run(R)
    spread = noise_spread(run, A, R)
    spread["eflx_fgr"] = spread["eflx_fgr"] + fgr_rounding_bound(R)
    out = sorted({n for (n, k, t, u) in abi.SOILWATER_FIELDS + abi.SOILTEMP_FIELDS if u != "in"})
    errs, bad = compare(P, R, out, 1e-9, spread)
    assert not bad, {k: errs[k] for k in bad}
