"""Drift of the batched engine against the oracle over a simulated year
(17,520 steps of 1800 s), checkpointed monthly, with the reference's balance
checks on every column.

Only SoilWater and SoilTemperature (and CanopyFluxes) are on this path, so a
long run is physical only where they close the budgets by themselves: the
water table is prognostic only through WaterTable, melted snow layers are
removed only by SnowHydrology, and negative soil liquid is repaired only by
the drainage routines -- all outside the path.  The year therefore runs on
snow-free columns without infiltration or root sink, whose soil water relaxes
toward the Zeng-Decker equilibrium profile (the steady state of SoilWater),
under constant radiative forcing on bare ground (some columns settle below
freezing, so Phasechange is exercised).  The full soil + canopy step runs 30 days on
snow-free columns (transpiration with a fixed btran dries the soil over
longer runs).  With the CLM5-default step -- the default hydrology's
infiltration, drainage and lateral flow around the moisture-form SoilWater,
the root moisture stress and the soil resistance following the soil state --
workload columns with transpiration and infiltration stay physical for a
year and run it in full (snow layers taken away: their removal after
melting is SnowHydrology's, outside the path)."""
import copy
import json
import os

import numpy as np
import pytest

from ctsm_gb300 import abi, balance, inputs, full_inputs as fi
from oracle.steps import full_steps

pytestmark = pytest.mark.gpu
LS = -abi.NLEVSNO + 1
PER_MONTH = 1460


def year_columns(ncol, seed):
    A, npatch = inputs.soil_columns(ncol, seed=seed, snow=False, nbedrock=(3, 20), forcing="full", npatch_max=4)
    r = np.random.Generator(np.random.Philox(seed + 1))
    for j in range(1, abi.NLEVGRND + 1):
        row = j - LS
        A["t_soisno"][row] = np.maximum(A["t_soisno"][row], 278.0)
        A["h2osoi_liq"][row] += A["h2osoi_ice"][row]
        A["h2osoi_ice"][row] = 0.0
    A["t_grnd"][:] = A["t_soisno"][1 - LS]
    A["t_h2osfc"][:] = A["t_grnd"]
    inputs.refresh_h2osoi_vol(A)
    A["qflx_infl"][:] = 0.0
    A["qflx_rootsoi"][:] = 0.0
    A["frac_veg_nosno"][:] = 0
    A["forc_lwrad"][:] = r.uniform(320.0, 420.0, ncol)
    A["sabg"][:] = r.uniform(50.0, 250.0, npatch)
    A["sabg_soil"][:] = A["sabg"]
    A["sabg_snow"][:] = A["sabg"]
    A["sabg_lyr"][:] = 0.0
    A["sabg_lyr"][1 - LS] = A["sabg"]
    # snow- and surface-water-free bare ground: the ground fluxes and their
    # soil components are the same flux (SoilFluxesMod.F90 weights them by
    # frac_sno_eff and frac_h2osfc, both 0 here); no canopy longwave
    sh = r.uniform(-20.0, 60.0, npatch)
    ev = r.uniform(0.0, 2e-5, npatch)
    for k in ("eflx_sh_grnd", "eflx_sh_snow", "eflx_sh_soil", "eflx_sh_h2osfc"):
        A[k][:] = sh
    for k in ("qflx_evap_soi", "qflx_ev_snow", "qflx_ev_soil", "qflx_ev_h2osfc"):
        A[k][:] = ev
    A["dlrad"][:] = 0.0
    A["eflx_bot"][:] = 0.0
    return A, npatch


def _soil_steps_oracle(A, npatch, n):
    import ctypes as C
    from oracle import oracle as orc
    L = orc.lib()
    ncol = A["zwt"].shape[0]
    b = abi.Bounds(1, ncol, 1, npatch)
    f = np.arange(1, ncol + 1, dtype=np.int32)
    fp = f.ctypes.data_as(C.POINTER(C.c_int32))
    for _ in range(n):
        sw = abi.make_io(abi.SoilWaterIO, abi.SOILWATER_FIELDS, A, ncol)
        assert L.oracle_soilwater(C.byref(b), ncol, fp, C.byref(sw), 6.0, 1800.0) == 0
        st = abi.make_io(abi.SoilTempIO, abi.SOILTEMP_FIELDS, A, ncol, npatch)
        assert L.oracle_soiltemperature(C.byref(b), ncol, fp, C.byref(st), 1800.0, 0) == 0
        inputs.refresh_h2osoi_vol(A)


def _diffs(G, R):
    soil = slice(1 - LS, None)
    return {"dT_max_K": float(np.abs(G["t_soisno"][soil] - R["t_soisno"][soil]).max()),
            "dliq_max_kg_m2": float(np.abs(G["h2osoi_liq"][soil] - R["h2osoi_liq"][soil]).max()),
            "dqcharge_max": float(np.abs(G["qcharge"] - R["qcharge"]).max())}


def test_year_soil_step_drift_and_balance(gpu_lib):
    from ctsm_gb300.engine import SoilBatch
    A, npatch = year_columns(512, seed=91)
    G, R = copy.deepcopy(A), copy.deepcopy(A)
    b = SoilBatch(G, npatch, balance=True)
    months = []
    for m in range(12):
        b.run(PER_MONTH)
        b.sync()
        b.download()
        _soil_steps_oracle(R, npatch, PER_MONTH)
        d = _diffs(G, R)
        d["T_range"] = [float(G["t_soisno"][1 - LS:].min()), float(G["t_soisno"][1 - LS:].max())]
        months.append(d)
    h2o, soi, _, _ = b.balance()
    b.close()
    print(json.dumps({"months": months, "errh2o_max": float(h2o.max()), "errsoi_max": float(soi.max()),
                      "soi_warn_cols": int((soi > balance.ERRSOI_WARNING).sum()),
                      "h2o_warn_cols": int((h2o > balance.H2O_WARNING_THRESH).sum())}))
    assert all(np.isfinite(list(d.values())[:3]).all() for d in months)
    # Bounded: levels that sit at the freezing point switch between melting
    # and freezing on an ulp of temperature (Phasechange's imelt test), so
    # the two runs part by up to one step's phase change at such levels and
    # the dissipative solve then pulls them together again.  No month may
    # exceed half a kelvin or 1 kg/m2 of liquid, and the year ends no worse
    # than its first quarter.
    for d in months:
        assert d["dT_max_K"] < 0.5 and d["dliq_max_kg_m2"] < 1.0, d
    assert months[-1]["dT_max_K"] <= max(d["dT_max_K"] for d in months[:3])
    assert months[-1]["dliq_max_kg_m2"] <= max(d["dliq_max_kg_m2"] for d in months[:3])
    # the reference's balance thresholds on every column, every checked step
    assert h2o.max() < balance.ERROR_THRESH and soi.max() < balance.ERRSOI_STOP


def test_month_full_step_drift_and_balance(gpu_lib):
    from ctsm_gb300.engine import SoilBatch
    A, npatch, ngrid, rootr = fi.full_state(384, seed=93)
    keep = A["snl"] == 0
    assert keep.sum() > 20
    G, R = copy.deepcopy(A), copy.deepcopy(A)
    b = SoilBatch(G, npatch, canopy=True, ngrid=ngrid, rootr=rootr, balance=True)
    out = []
    for k in range(3):                    # 3 x 10 days
        b.run(480)
        b.sync()
        b.download()
        full_steps(R, npatch, ngrid, rootr, 480)
        cols = np.nonzero(keep)[0]
        out.append({"dT_max_K": float(np.abs(G["t_soisno"][1 - LS:, cols] - R["t_soisno"][1 - LS:, cols]).max()),
                    "dtveg_max_K": float(np.abs(G["t_veg"] - R["t_veg"]).max()),
                    "niter_mismatch": int((G["num_iter"] != R["num_iter"]).sum())})
    h2o, soi, _, _ = b.balance()
    b.close()
    print(json.dumps({"tenths": out, "errh2o_max_snowfree": float(h2o[keep].max()),
                      "errsoi_max_snowfree": float(soi[keep].max())}))
    for d in out:
        assert d["dT_max_K"] < 0.5, d
    assert h2o[keep].max() < balance.ERROR_THRESH and soi[keep].max() < balance.ERRSOI_STOP


def snow_free(A):
    """The workload columns without snow layers (full_inputs.snow_free)."""
    return fi.snow_free(A)


def test_year_clm5_step_drift(gpu_lib):
    """A simulated year (17,520 steps) of the CLM5-default step on
    workload-derived columns: CanopyFluxes transpiring through the root sink,
    infiltration of rain through the default hydrology's infiltration chain,
    drainage and lateral flow, root moisture stress and the soil resistance
    following the soil state, the moisture-form SoilWater.  GPU against the
    oracle in lock-step, compared monthly: bounded drift, every state finite
    and physical (no negative soil liquid, temperatures in range)."""
    from ctsm_gb300 import canopy
    from ctsm_gb300.engine import SoilBatch
    A, npatch, ngrid, rootr, member_col, f = fi.ensemble(1, seed=33, cols=(300, 300), clm5=True)
    snow_free(A)
    ncol = A["zwt"].shape[0]
    nml = abi.soilwater_movement_nml(1)
    gpu_lib.set_soilwater_movement(nml)
    gpu_lib.set_soilhydrology_params()
    gpu_lib.set_soil_resistance()
    canopy.set_params()
    cols = np.arange(1, ncol + 1, dtype=np.int32)
    kw = dict(medlyn_per_patch=True, soilfluxes=True, rootmoist=True, swm=nml,
              soilresis=[(cols, abi.SoilResistanceParams(1, fi.D_MAX * f["d_max"][0], 0.8))],
              hydro=[(cols, abi.SoilHydrologyParams(0.01, 1.0, fi.BASEFLOW_SCALAR * f["baseflow_scalar"][0], 1.0e-5,
                                                    6.0, fi.FFF * f["fff"][0], 0.4, 0.13, 1))])
    try:
        G, R = copy.deepcopy(A), copy.deepcopy(A)
        b = SoilBatch(G, npatch, canopy=True, ngrid=ngrid, per_patch_medlyn=True, soilfluxes=True, rootmoist=True,
                      soilresis=True, hydrology=True, per_column_hydrology=True)
        months = []
        for m in range(12):
            b.run(PER_MONTH)
            b.sync()
            b.download()
            full_steps(R, npatch, ngrid, rootr, PER_MONTH, **kw)
            soil = slice(1 - LS, None)
            d = {"dT_max_K": float(np.abs(G["t_soisno"][soil] - R["t_soisno"][soil]).max()),
                 "dliq_max_kg_m2": float(np.abs(G["h2osoi_liq"][1 - LS:1 - LS + abi.NLEVSOI] -
                                                R["h2osoi_liq"][1 - LS:1 - LS + abi.NLEVSOI]).max()),
                 "dzwt_max_m": float(np.abs(G["zwt"] - R["zwt"]).max()),
                 "dtveg_max_K": float(np.abs(G["t_veg"] - R["t_veg"]).max()),
                 "T_range": [float(G["t_soisno"][soil].min()), float(G["t_soisno"][soil].max())],
                 "liq_min": float(G["h2osoi_liq"][1 - LS:1 - LS + abi.NLEVSOI].min()),
                 "zwt_range": [float(G["zwt"].min()), float(G["zwt"].max())]}
            months.append(d)
            for S in (G, R):
                assert np.isfinite(S["t_soisno"]).all() and np.isfinite(S["h2osoi_liq"]).all() and \
                    np.isfinite(S["t_veg"]).all(), m
        b.close()
        print(json.dumps({"months": months}))
        for d in months:
            # both runs stay physical: no negative soil liquid, temperatures
            # inside the range the forcing allows
            assert d["liq_min"] > -1e-6 and 200.0 < d["T_range"][0] and d["T_range"][1] < 350.0, d
            # bounded drift: levels at the freezing point part by one step's
            # phase change at most and the dissipative solve pulls them back;
            # the water table moves by whole layers and the drainage and
            # lateral flows by the water above thresholds (watmin, saturation),
            # so liquid differs by a few mm where one run crossed a threshold a
            # step before the other -- fluctuating month to month, not growing
            assert d["dT_max_K"] < 0.5 and d["dliq_max_kg_m2"] < 2.0 and d["dtveg_max_K"] < 0.5, d
        assert months[-1]["dT_max_K"] <= max(x["dT_max_K"] for x in months[:3]) + 0.05
        assert np.mean([x["dliq_max_kg_m2"] for x in months[-6:]]) < 2.0 * np.mean([x["dliq_max_kg_m2"]
                                                                                    for x in months[:6]])
    finally:
        gpu_lib.set_soilwater_movement(abi.soilwater_movement_nml(0, use_bedrock=0))
