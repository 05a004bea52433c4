"""The batched resident engine against the oracle stepped the same way:
SoilWater, SoilTemperature, h2osoi_vol refresh, for several steps."""
import copy
import ctypes as C

import numpy as np
import pytest

from ctsm_gb300 import abi, inputs
from tests.parity import compare, noise_spread

pytestmark = pytest.mark.gpu
DT = 1800.0
STATE = ["h2osoi_liq", "h2osoi_ice", "t_soisno", "t_grnd", "t_h2osfc", "h2osoi_vol", "qcharge", "qflx_deficit",
         "xmf", "snow_depth", "int_snow", "h2osno_no_layers"]


def oracle_steps(A, npatch, nsteps):
    from oracle import oracle as orc
    L = orc.lib()
    ncol = A["zwt"].shape[0]
    b = abi.Bounds(1, ncol, 1, npatch)
    filt = np.arange(1, ncol + 1, dtype=np.int32)
    fp = filt.ctypes.data_as(C.POINTER(C.c_int32))
    sw = abi.make_io(abi.SoilWaterIO, abi.SOILWATER_FIELDS, A, ncol)
    st = abi.make_io(abi.SoilTempIO, abi.SOILTEMP_FIELDS, A, ncol, npatch)
    for _ in range(nsteps):
        assert L.oracle_soilwater(C.byref(b), ncol, fp, C.byref(sw), 6.0, DT) == 0
        assert L.oracle_soiltemperature(C.byref(b), ncol, fp, C.byref(st), DT, 0) == 0
        inputs.refresh_h2osoi_vol(A)


@pytest.mark.parametrize("nsteps", [1, 6])
def test_batch_matches_oracle(gpu_lib, nsteps):
    from ctsm_gb300.engine import SoilBatch
    A, npatch = inputs.soil_columns(6000, seed=77, snow=True, nbedrock=(3, 20), forcing="full", npatch_max=4,
                                    h2osfc=True)
    R = copy.deepcopy(A)
    oracle_steps(R, npatch, nsteps)
    G = copy.deepcopy(A)
    b = SoilBatch(G, npatch, dtime=DT)
    b.run(nsteps)
    b.sync()
    b.download()
    b.close()
    # a multi-step comparison accumulates ulp-level differences through the
    # state; state variables stay at 1e-9, the cancellation diagnostics are
    # judged against the oracle's own spread under libm noise over the same steps
    spread = noise_spread(lambda B: oracle_steps(B, npatch, nsteps), A, R, fields=("xmf",))
    errs, bad = compare(G, R, STATE, 1e-9, spread)
    assert not bad, {k: errs[k] for k in bad}


def test_batch_autotune_restores_state(gpu_lib):
    from ctsm_gb300.engine import SoilBatch
    A, npatch = inputs.soil_columns(4096, seed=5, snow=True, nbedrock=(3, 20))
    G1 = copy.deepcopy(A)
    b1 = SoilBatch(G1, npatch)
    blk = b1.autotune(trial_steps=1)
    assert blk in (64, 128, 256)
    b1.run(3)
    b1.sync()
    b1.download()
    b1.close()
    G2 = copy.deepcopy(A)
    b2 = SoilBatch(G2, npatch)
    b2.set_block(blk)
    b2.run(3)
    b2.sync()
    b2.download()
    b2.close()
    for k in STATE:
        np.testing.assert_array_equal(G1[k], G2[k])


def test_batch_order_invariance(gpu_lib):
    """The same column gives identical results whatever batch it is in and
    wherever it sits (the reference's ERP idea: results independent of the
    decomposition)."""
    from ctsm_gb300.engine import SoilBatch
    A, npatch = inputs.soil_columns(2048, seed=6, snow=True, nbedrock=(3, 20))
    G = copy.deepcopy(A)
    b = SoilBatch(G, npatch)
    b.run(2)
    b.sync()
    b.download()
    b.close()
    sub = np.arange(100, 612)
    S = {}
    for k, v in A.items():
        S[k] = np.ascontiguousarray(v[..., sub][..., ::-1])
    S["col_patchi"] = np.arange(1, len(sub) + 1, dtype=np.int32)
    b = SoilBatch(S, len(sub))
    b.run(2)
    b.sync()
    b.download()
    b.close()
    for k in ("h2osoi_liq", "t_soisno", "qcharge"):
        np.testing.assert_array_equal(S[k], G[k][..., sub][..., ::-1])


def test_autotune_orders_and_blocks_leave_results_unchanged(gpu_lib):
    """ctsmg_batch_autotune2 times every (column order, threads per block)
    candidate and moves the resident columns into the chosen order; a tuned
    batch then steps to the same bits as an untuned one (results are returned
    in the caller's column order either way), and each forced order gives the
    same bits too.  The caller's order is the slowest of the four: sorting by
    layer counts is what lets a warp's lanes run level loops of equal length."""
    from ctsm_gb300.engine import SoilBatch
    A, npatch = inputs.soil_columns(20000, seed=78, snow=True, nbedrock=(3, 20), forcing="full", npatch_max=3,
                                    h2osfc=True)
    U = copy.deepcopy(A)
    b = SoilBatch(U, npatch)
    b.run(3)
    b.sync()
    b.download()
    b.close()
    T = copy.deepcopy(A)
    b = SoilBatch(T, npatch, balance=True)
    tuned = b.tune(trial_steps=1)
    assert tuned["block"] in (64, 128, 256) and len(tuned["ms_per_step"]) == 4
    assert all(len(v) == 3 and min(v.values()) > 0 for v in tuned["ms_per_step"].values())
    b.run(3)
    b.sync()
    b.download()
    h2o, soi, _, _ = b.balance()
    b.close()
    for k in STATE + ["t_soisno", "qin", "qout", "fact"]:
        assert np.array_equal(T[k], U[k], equal_nan=True), k
    assert np.isfinite(h2o).all() and np.isfinite(soi).all()
    t = tuned["ms_per_step"]
    assert min(t["caller"].values()) > min(t["snl,nbedrock,zwt"].values())
