"""The root-sink drop-in (ctsmg_root_sink, replacing
Compute_EffecRootFrac_And_VertTranSink_Default, SoilWaterPlantSinkMod.F90:332-420)
against the oracle: a filter subset with offset bounds, 1-4 patches per
column, a column without transpiration, the column transpiration given and
NULL."""
import copy
import ctypes as C

import numpy as np
import pytest

from ctsm_gb300 import abi
from tests.parity import compare
from tests.test_rootsink_cpu import case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tran_col", [True, False])
def test_root_sink_matches_oracle(gpu_lib, tran_col):
    from oracle import oracle as orc
    A, npatch, filt, b = case(ncol=20000, seed=9)
    ncol = A["col_patchi"].shape[0]
    G, R = copy.deepcopy(A), copy.deepcopy(A)
    gpu_lib.RootSink(b, len(filt), filt, G, tran_col=tran_col)
    fields = [x for x in abi.ROOTSINK_FIELDS if tran_col or x[0] != "qflx_tran_veg_col"]
    io = abi.make_io(abi.RootSinkIO, fields, R, ncol, npatch)
    assert orc.lib().oracle_root_sink(C.byref(b), len(filt), filt.ctypes.data_as(C.POINTER(C.c_int32)),
                                      C.byref(io)) == 0
    errs, bad = compare(G, R, ["rootr_col", "qflx_rootsoi"], 1e-12)
    assert not bad, errs
    untouched = np.setdiff1d(np.arange(ncol), filt - b.begc)
    assert (G["qflx_rootsoi"][:, untouched] == -7.0).all()
