"""The reference's balance thresholds on every column of the batched engine
(BalanceCheckMod.F90: water error warning 1e-9 mm / stop 1e-5 mm, :506,626;
soil energy errsoi warning 1e-5 / stop 1e-4 W/m2, :1105,1111), after the
first skip_steps steps (:91)."""
import copy

import numpy as np
import pytest

from ctsm_gb300 import balance, inputs, full_inputs as fi

pytestmark = pytest.mark.gpu


def _run(A, npatch, nsteps, **kw):
    from ctsm_gb300.engine import SoilBatch
    G = copy.deepcopy(A)
    b = SoilBatch(G, npatch, balance=True, **kw)
    b.run(nsteps)
    b.sync()
    out = b.balance()
    b.close()
    return out


def test_soil_batch_balances_close():
    """Uneven-column workload (SoilWater then SoilTemperature), 12 steps."""
    A, npatch = inputs.soil_columns(8192, seed=61, snow=True, nbedrock=(3, 20))
    h2o_max, soi_max, h2o_last, soi_last = _run(A, npatch, 12)
    assert np.isfinite(h2o_max).all() and np.isfinite(soi_max).all()
    assert h2o_max.max() < balance.H2O_WARNING_THRESH, h2o_max.max()
    assert soi_max.max() < balance.ERRSOI_WARNING, soi_max.max()
    assert (h2o_max > 0).any()          # the check ran on the steps after skip_steps


def test_full_step_balances_close():
    """Full soil + canopy step (driver order): the fluxes SoilTemperature
    receives come from CanopyFluxes, so errsoi tests their consistency."""
    A, npatch, ngrid, rootr = fi.full_state(3000, seed=62)
    h2o_max, soi_max, _, _ = _run(A, npatch, 8, canopy=True, ngrid=ngrid, rootr=rootr)
    assert h2o_max.max() < balance.H2O_WARNING_THRESH, h2o_max.max()
    assert soi_max.max() < balance.ERRSOI_WARNING, soi_max.max()


def test_balance_state_matches_numpy_water_budget():
    """The device water error equals the same budget evaluated on the state
    the engine returns (independent evaluation on the host)."""
    from ctsm_gb300.engine import SoilBatch
    A, npatch = inputs.soil_columns(2048, seed=63, snow=True, nbedrock=(3, 20))
    G = copy.deepcopy(A)
    b = SoilBatch(G, npatch, balance=True, skip_steps=0)
    b.run(1)
    b.sync()
    b.download()
    _, _, h2o_last, _ = b.balance()
    b.close()
    LS = -inputs.NLEVSNO + 1

    def water(S):
        w = S["h2osfc"] + S["h2osno_no_layers"]
        for j in range(LS, inputs.NLEVSOI + 1):
            act = j >= S["snl"] + 1
            w = w + np.where(act, S["h2osoi_liq"][j - LS] + S["h2osoi_ice"][j - LS], 0.0)
        return w
    deep = A["zwt"] > A["zi"][inputs.NLEVSOI + inputs.NLEVSNO]
    net = (A["qflx_infl"] - A["qflx_rootsoi"].sum(axis=0) - np.where(deep, G["qcharge"], 0.0)) * 1800.0
    err = (water(G) - water(A)) - net
    np.testing.assert_allclose(h2o_last, err, atol=1e-11)
