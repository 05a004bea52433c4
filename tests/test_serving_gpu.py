"""Serving pool on the GPU: a request gives bit-identical results alone, in a
mix of requests admitted while it runs, and as a plain batch; it matches the
oracle; admission waits for free slots; a request stopped early holds the
state of the steps it ran; a request larger than the free ranges is refused
without changing the pool."""
import copy

import numpy as np
import pytest

from ctsm_gb300 import serving
from oracle.steps import full_steps
from tests.parity import compare, noise_spread, evap_veg_rounding_bound

pytestmark = pytest.mark.gpu
OUT = ["h2osoi_liq", "h2osoi_ice", "t_soisno", "t_grnd", "h2osoi_vol", "t_veg", "eflx_sh_veg", "qflx_evap_veg",
       "qflx_tran_veg", "cgrnd", "dlrad", "psnsun", "psnsha", "rssun", "rssha", "liqcan", "snocan", "qcharge",
       "eflx_sh_grnd", "qflx_evap_soi", "xmf", "num_iter", "qflx_rootsoi", "smp_l", "hk_l", "eflx_fgr", "imelt",
       "t_h2osfc", "qin", "qout", "fv", "u10"]
CANCEL = ("liqcan", "snocan", "eflx_sh_grnd", "qflx_evap_soi", "xmf")


def _clone(q, arrival=None):
    Q = copy.copy(q)
    Q.state = {k: np.array(v, copy=True) for k, v in q.state.items()}
    Q.rootr = q.rootr.copy()
    Q.extra = {}
    if arrival is not None:
        Q.arrival = arrival
    return Q


def _batch(q, nsteps):
    from ctsm_gb300.engine import SoilBatch
    G = {k: np.array(v, copy=True) for k, v in q.state.items()}
    b = SoilBatch(G, q.npatch, canopy=True, ngrid=q.ngrid, rootr=q.rootr, per_patch_medlyn=True)
    b.run(nsteps)
    b.sync()
    b.download()
    b.close()
    return G


def _same(a, b, fields=OUT):
    for k in fields:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_request_alone_mix_and_batch_identical(gpu_lib):
    q = serving.make_request(0, 777, 300, 10, pinned=False)
    alone = _clone(q)
    pool = serving.Pool(col_capacity=4096)
    st = serving.serve(pool, [alone], tick_clock=True)
    pool.close()
    assert st["completed"] == 1 and alone.steps_done == 10
    mine = _clone(q, arrival=3)
    mix = [serving.make_request(1, 11, 900, 14, arrival=0, pinned=False), mine,
           serving.make_request(2, 12, 50, 4, arrival=4, pinned=False),
           serving.make_request(3, 13, 1200, 6, arrival=5, pinned=False),
           serving.make_request(4, 14, 1, 9, arrival=7, pinned=False)]
    pool = serving.Pool(col_capacity=4096)
    st = serving.serve(pool, mix, tick_clock=True)
    pool.close()
    assert st["completed"] == 5
    assert st["max_running_columns"] >= 900 + 300 + 50 + 1200      # the request shared ticks with others
    _same(alone.state, mine.state)
    _same(alone.state, _batch(q, 10))


def test_pool_request_matches_oracle(gpu_lib):
    q = serving.make_request(0, 4242, 160, 3, pinned=False)
    A = {k: np.array(v, copy=True) for k, v in q.state.items()}
    R = copy.deepcopy(A)
    run = lambda B: full_steps(B, q.npatch, q.ngrid, q.rootr, 3, medlyn_per_patch=True)
    run(R)
    G = _clone(q)
    pool = serving.Pool(col_capacity=512)
    serving.serve(pool, [G], tick_clock=True)
    pool.close()
    spread = noise_spread(run, A, R, fields=CANCEL, input_ulps=4)
    for k in ("liqcan", "snocan"):
        spread[k] = spread[k] + 1e-9 * (np.abs(A["liqcan"]) + np.abs(A["snocan"]))
    errs, bad = compare(G.state, R, OUT[:22], 1e-9, spread)
    assert not bad, {k: errs[k] for k in bad}


def test_admission_waits_for_free_slots(gpu_lib):
    a = serving.make_request(0, 21, 700, 5, arrival=0, pinned=False)
    b = serving.make_request(1, 22, 600, 3, arrival=1, pinned=False)
    c = serving.make_request(2, 23, 200, 2, arrival=1, pinned=False)
    b_alone = _clone(b)
    pool = serving.Pool(col_capacity=1000)
    st = serving.serve(pool, [a, b, c], tick_clock=True)
    pool.close()
    assert st["completed"] == 3
    assert b.t_admit >= a.t_done and c.t_admit >= b.t_admit     # first in, first out behind the blocked request
    pool = serving.Pool(col_capacity=1000)
    serving.serve(pool, [b_alone], tick_clock=True)
    pool.close()
    _same(b.state, b_alone.state)


def test_stopped_request_and_refusal(gpu_lib):
    q = serving.make_request(0, 99, 250, 10, pinned=False)
    G = _clone(q)
    pool = serving.Pool(col_capacity=600)
    before = pool.largest_free()
    big = serving.make_request(1, 98, 601, 2, pinned=False)
    assert pool.admit(big) is None and pool.largest_free() == before
    pool.admit(G)
    for _ in range(4):
        pool.tick()
    assert pool.evict(G) == 4
    pool.sync()
    assert pool.largest_free() == before
    pool.close()
    _same(G.state, _batch(q, 4))


HYD_DEFAULTS = dict(aq_sp_yield_min=0.01, n_baseflow=1.0, baseflow_scalar=1.0e-2, perched_baseflow_scalar=1.0e-5,
                    e_ice=6.0, fff=0.5, pc=0.4, mu=0.13, h2osfcflag=1)


def test_rootmoist_pool_matches_batch_and_oracle(gpu_lib):
    """A pool with the root moisture stress (btran and rootr from the soil
    state at the start of every tick, CanopyFluxesMod.F90:709) and the
    aquifer-layer hydrology around the Zeng-Decker SoilWater (saturated
    excess, infiltration, water table, drainage): a snow-free request alone
    in the pool equals the resident batch with both bit for bit, and the
    oracle stepped the same way within the parity tolerance; the stress and
    hydrology outputs come back with the request."""
    from ctsm_gb300 import abi
    from ctsm_gb300.engine import SoilBatch
    gpu_lib.set_soilhydrology_params(**HYD_DEFAULTS)
    q = serving.make_request(0, 515, 240, 4, pinned=False, physical=True)
    assert (q.state["snl"] == 0).all() and "rootfr" in q.state and "wa" in q.state
    A = {k: np.array(v, copy=True) for k, v in q.state.items()}
    G = _clone(q)
    pool = serving.Pool(col_capacity=1024, rootmoist=True, hydrology=True)
    st = serving.serve(pool, [G], tick_clock=True)
    pool.close()
    assert st["completed"] == 1 and G.steps_done == 4
    B = {k: np.array(v, copy=True) for k, v in q.state.items()}
    b = SoilBatch(B, q.npatch, canopy=True, ngrid=q.ngrid, per_patch_medlyn=True, rootmoist=True, hydrology=True)
    b.run(4)
    b.sync()
    b.download()
    b.close()
    _same(G.state, B, OUT + ["btran", "rootr", "rresis", "zwt", "wa", "qflx_drain", "qflx_infl"])
    R = copy.deepcopy(A)
    cols = np.arange(1, q.ncol + 1, dtype=np.int32)
    par = abi.SoilHydrologyParams(*HYD_DEFAULTS.values())
    run = lambda S: full_steps(S, q.npatch, q.ngrid, q.rootr, 4, medlyn_per_patch=True, rootmoist=True,
                               hydro=[(cols, par)])
    run(R)
    spread = noise_spread(run, A, R, fields=CANCEL + ("qflx_evap_veg", "qflx_drain"), input_ulps=4)
    for k in ("liqcan", "snocan"):
        spread[k] = spread[k] + 1e-9 * (np.abs(A["liqcan"]) + np.abs(A["snocan"]))
    # near saturation the sign of efpot is set by rounding (see parity.evap_veg_rounding_bound)
    spread["qflx_evap_veg"] = spread["qflx_evap_veg"] + evap_veg_rounding_bound(R)
    errs, bad = compare(G.state, R, OUT[:22] + ["btran", "zwt", "wa", "qflx_drain"], 1e-9, spread)
    assert not bad, {k: errs[k] for k in bad}


def test_physical_stream_stays_finite(gpu_lib):
    """Year-long requests through the pool with the root moisture stress and
    the hydrology stay in the physical domain: 6 requests of 40..400
    columns, 17,520 steps (a simulated year) each, every final state finite,
    no negative soil liquid, temperatures in range."""
    gpu_lib.set_soilhydrology_params(**HYD_DEFAULTS)
    reqs = serving.request_stream(6, 0.0, seed=99, cols=(40, 400), steps=(17520, 17520), pinned=False,
                                  physical=True)
    pool = serving.Pool(col_capacity=4096, rootmoist=True, hydrology=True)
    st = serving.serve(pool, reqs, tick_clock=True)
    pool.close()
    assert st["completed"] == 6
    for q in reqs:
        A = q.state
        assert q.extra["nonfinite_columns"] == 0, q.rid
        soil = A["h2osoi_liq"][serving.abi.NLEVSNO:serving.abi.NLEVSNO + serving.abi.NLEVSOI]
        assert soil.min() >= -1e-9, (q.rid, float(soil.min()))
        T = A["t_soisno"][serving.abi.NLEVSNO:]
        assert 200.0 < T.min() and T.max() < 350.0, (q.rid, float(T.min()), float(T.max()))
