"""The oracle's Compute_EffecRootFrac_And_VertTranSink_Default
(SoilWaterPlantSinkMod.F90:332-420) against an independent numpy evaluation
of the same sums, with 1-4 patches per column, columns without transpiration
(no quotient) and a filter subset with offset bounds."""
import ctypes as C

import numpy as np

from ctsm_gb300 import abi


def case(ncol=300, seed=5, begc=11, begp=4):
    r = np.random.Generator(np.random.Philox(seed))
    npc = r.integers(1, 5, ncol).astype(np.int32)
    npatch = int(npc.sum())
    A = {"col_patchi": (np.concatenate([[0], np.cumsum(npc)[:-1]]) + begp).astype(np.int32),
         "col_npatches": npc,
         "wtcol": np.concatenate([r.dirichlet(np.ones(k)) for k in npc]),
         "qflx_tran_veg": r.uniform(0.0, 1e-4, npatch),
         "qflx_tran_veg_col": r.uniform(0.0, 1e-4, ncol),
         "rootr": np.ascontiguousarray(r.uniform(0.0, 0.2, (abi.NLEVGRND, npatch))),
         "rootr_col": np.full((abi.NLEVGRND, ncol), -7.0),
         "qflx_rootsoi": np.full((abi.NLEVSOI, ncol), -7.0)}
    A["qflx_tran_veg"][A["col_patchi"][3] - begp: A["col_patchi"][3] - begp + npc[3]] = 0.0   # column 4: none
    keep = np.union1d(r.permutation(ncol)[: ncol - 40], [3])          # column 4 always filtered
    filt = (keep + begc).astype(np.int32)
    return A, npatch, filt, abi.Bounds(begc, begc + ncol - 1, begp, begp + npatch - 1)


def numpy_sink(A, filt, b, tran_col):
    R = {k: v.copy() for k, v in A.items()}
    for cg in filt:
        c = cg - b.begc
        ps = np.arange(A["col_patchi"][c] - b.begp, A["col_patchi"][c] - b.begp + A["col_npatches"][c])
        w = A["qflx_tran_veg"][ps] * A["wtcol"][ps]
        temp = w.sum()
        rc = (A["rootr"][:abi.NLEVSOI, ps] * w).sum(axis=1)
        if temp != 0.0:
            rc = rc / temp
        R["rootr_col"][:abi.NLEVSOI, c] = rc
        R["qflx_rootsoi"][:, c] = rc * (A["qflx_tran_veg_col"][c] if tran_col else temp)
    return R


def test_oracle_root_sink_matches_numpy():
    from oracle import oracle as orc
    L = orc.lib()
    for tran_col in (True, False):
        A, npatch, filt, b = case()
        ncol = A["col_patchi"].shape[0]
        fields = [x for x in abi.ROOTSINK_FIELDS if tran_col or x[0] != "qflx_tran_veg_col"]
        io = abi.make_io(abi.RootSinkIO, fields, A, ncol, npatch)
        R = numpy_sink(A, filt, b, tran_col)
        assert L.oracle_root_sink(C.byref(b), len(filt), filt.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(io)) == 0
        for k in ("rootr_col", "qflx_rootsoi"):
            np.testing.assert_allclose(A[k], R[k], rtol=1e-13, atol=1e-25)
        untouched = np.setdiff1d(np.arange(ncol), filt - b.begc)
        assert (A["qflx_rootsoi"][:, untouched] == -7.0).all()
        assert (A["qflx_rootsoi"][:, 3] == 0.0).all()
