"""The full soil + canopy step (driver order) and the perturbed-parameter
ensemble in the batched engine, against the oracle stepped the same way."""
import copy

import numpy as np
import pytest

from ctsm_gb300 import full_inputs as fi
from oracle.steps import full_steps
from tests.parity import compare, noise_spread, evap_veg_rounding_bound

pytestmark = pytest.mark.gpu
STATE = ["h2osoi_liq", "h2osoi_ice", "t_soisno", "t_grnd", "h2osoi_vol", "t_veg", "eflx_sh_veg", "qflx_evap_veg",
         "qflx_tran_veg", "cgrnd", "dlrad", "psnsun", "psnsha", "rssun", "rssha", "liqcan", "snocan", "qcharge",
         "eflx_sh_grnd", "qflx_evap_soi", "xmf", "num_iter"]
CANCEL = ("liqcan", "snocan", "eflx_sh_grnd", "qflx_evap_soi", "xmf")


def _run(A, npatch, ngrid, rootr, nsteps, per_patch=False):
    from ctsm_gb300.engine import SoilBatch
    G = copy.deepcopy(A)
    b = SoilBatch(G, npatch, canopy=True, ngrid=ngrid, rootr=rootr, per_patch_medlyn=per_patch)
    b.run(nsteps)
    b.sync()
    b.download()
    b.close()
    return G


@pytest.mark.parametrize("nsteps", [1, 3])
def test_full_step_matches_oracle(gpu_lib, nsteps):
    A, npatch, ngrid, rootr = fi.full_state(2500, seed=31)
    R = copy.deepcopy(A)
    full_steps(R, npatch, ngrid, rootr, nsteps)
    G = _run(A, npatch, ngrid, rootr, nsteps)
    spread = noise_spread(lambda B: full_steps(B, npatch, ngrid, rootr, nsteps), A, R, fields=CANCEL, input_ulps=4)
    for k in ("liqcan", "snocan"):
        spread[k] = spread[k] + 1e-9 * (np.abs(A["liqcan"]) + np.abs(A["snocan"]))
    errs, bad = compare(G, R, STATE, 1e-9, spread)
    assert not bad, {k: errs[k] for k in bad}


def test_ensemble_members_match_oracle(gpu_lib):
    """Several members with perturbed Medlyn slope/intercept and organic-matter
    scale packed into one batch: each member's result equals the oracle's."""
    A, npatch, ngrid, rootr, member_col, factors = fi.ensemble(6, seed=4, cols=(200, 700))
    R = copy.deepcopy(A)
    full_steps(R, npatch, ngrid, rootr, 2, medlyn_per_patch=True)
    G = _run(A, npatch, ngrid, rootr, 2, per_patch=True)
    spread = noise_spread(lambda B: full_steps(B, npatch, ngrid, rootr, 2, medlyn_per_patch=True), A, R,
                          fields=CANCEL, input_ulps=4)
    for k in ("liqcan", "snocan"):
        spread[k] = spread[k] + 1e-9 * (np.abs(A["liqcan"]) + np.abs(A["snocan"]))
    errs, bad = compare(G, R, STATE, 1e-9, spread)
    assert not bad, {k: errs[k] for k in bad}
    assert len(np.unique(factors["medlynslope"])) == 6


def test_member_alone_equals_member_in_ensemble(gpu_lib):
    """A member run by itself gives bit-identical results to the same member
    packed with others (results do not depend on the batch around them)."""
    A, npatch, ngrid, rootr, member_col, factors = fi.ensemble(3, seed=9, cols=(150, 400))
    G = _run(A, npatch, ngrid, rootr, 2, per_patch=True)
    m = 1
    cols = np.nonzero(member_col == m)[0]
    pmask = np.isin(A["patch_column"] - 1, cols)
    pidx = np.nonzero(pmask)[0]
    S = {}
    for k, v in A.items():
        if v.shape[-1] == A["zwt"].shape[0]:
            S[k] = np.ascontiguousarray(v[..., cols])
        elif v.shape[-1] == npatch:
            S[k] = np.ascontiguousarray(v[..., pidx])
    S["col_patchi"] = (A["col_patchi"][cols] - pidx[0]).astype(np.int32)
    S["patch_column"] = (A["patch_column"][pidx] - cols[0]).astype(np.int32)
    S["patch_gridcell"] = S["patch_column"].copy()
    Gs = _run(S, len(pidx), len(cols), np.ascontiguousarray(rootr[:, pidx]), 2, per_patch=True)
    for k in ("t_soisno", "h2osoi_liq", "t_veg", "psnsun", "qcharge"):
        g = G[k][..., cols] if G[k].shape[-1] == A["zwt"].shape[0] else G[k][..., pidx]
        np.testing.assert_array_equal(Gs[k], g)


SF_OUT = ["eflx_soil_grnd", "eflx_sh_tot", "qflx_evap_tot", "eflx_lh_tot", "eflx_lwrad_out", "eflx_lwrad_net",
          "qflx_liqevap_from_top_layer", "qflx_solidevap_from_top_layer", "eflx_lh_grnd"]


def test_full_step_with_soilfluxes_matches_oracle(gpu_lib):
    """Driver order with SoilFluxes between SoilTemperature and SoilWater
    (clm_driver.F90:900,921,950) in the resident engine, against the oracle
    stepped the same way."""
    from ctsm_gb300.engine import SoilBatch
    A, npatch, ngrid, rootr = fi.full_state(2500, seed=34)
    fi.add_soilfluxes_fields(A, npatch, ngrid)
    R = copy.deepcopy(A)
    full_steps(R, npatch, ngrid, rootr, 3, soilfluxes=True)
    G = copy.deepcopy(A)
    b = SoilBatch(G, npatch, canopy=True, ngrid=ngrid, rootr=rootr, soilfluxes=True)
    b.run(3)
    b.sync()
    b.download()
    b.close()
    spread = noise_spread(lambda B: full_steps(B, npatch, ngrid, rootr, 3, soilfluxes=True), A, R,
                          fields=CANCEL + ("eflx_soil_grnd", "eflx_sh_tot", "eflx_lwrad_net"), input_ulps=4)
    for k in ("liqcan", "snocan"):
        spread[k] = spread[k] + 1e-9 * (np.abs(A["liqcan"]) + np.abs(A["snocan"]))
    errs, bad = compare(G, R, STATE + SF_OUT, 1e-9, spread)
    assert not bad, {k: errs[k] for k in bad}
    assert np.abs(G["errsoi_col"] - R["errsoi_col"]).max() < 1e-8
    assert np.abs(G["errsoi_col"]).max() < 1e-5          # the reference's errsoi warning threshold


def test_full_step_with_root_moisture_stress_matches_oracle(gpu_lib):
    """btran and rootr computed from the resident soil state at the start of
    every step (CanopyFluxesMod.F90:833-895) and fed to CanopyFluxes and the
    root sink, with SoilFluxes, over 3 steps."""
    from ctsm_gb300.engine import SoilBatch
    A, npatch, ngrid, rootr = fi.full_state(2500, seed=35)
    fi.add_soilfluxes_fields(A, npatch, ngrid)
    fi.add_rootmoist_fields(A, npatch, rootr, rng=np.random.Generator(np.random.Philox(36)))
    R = copy.deepcopy(A)
    full_steps(R, npatch, ngrid, None, 3, soilfluxes=True, rootmoist=True)
    G = copy.deepcopy(A)
    b = SoilBatch(G, npatch, canopy=True, ngrid=ngrid, soilfluxes=True, rootmoist=True)
    b.run(3)
    b.sync()
    b.download()
    b.close()
    assert (R["btran"] != A["btran"]).mean() > 0.9          # the stress really was recomputed
    # rresis = (eff/watsat)*(smp - smpsc)/(smpso - smpsc) cancels where the
    # suction nears smpsc, and smp ~ s^-bsw amplifies the state's rounding by
    # bsw: those fields (and the transpiration they scale) get the
    # conditioned test
    spread = noise_spread(lambda B: full_steps(B, npatch, ngrid, None, 3, soilfluxes=True, rootmoist=True), A, R,
                          fields=CANCEL + ("eflx_soil_grnd", "eflx_sh_tot", "eflx_lwrad_net", "rresis", "rootr",
                                           "btran", "qflx_evap_veg", "qflx_tran_veg"), input_ulps=4)
    for k in ("liqcan", "snocan"):
        spread[k] = spread[k] + 1e-9 * (np.abs(A["liqcan"]) + np.abs(A["snocan"]))
    # with btran = 0 (frozen or dry root zones) and a dry canopy,
    # qflx_evap_veg = min(rpp*efpot, 0) and efpot is a difference of
    # humidities (CanopyFluxesMod.F90:1336-1364) crossing zero at dew point:
    # its rounding, ~eps*qsat/dq ~ 1e-14 of the field's scale, decides the sign
    spread["qflx_evap_veg"] = spread["qflx_evap_veg"] + 1e-14 * np.abs(R["qflx_evap_veg"]).max()
    errs, bad = compare(G, R, STATE + SF_OUT + ["btran", "rootr", "rresis", "eff_porosity", "h2osoi_liqvol"], 1e-9,
                        spread)
    assert not bad, {k: errs[k] for k in bad}


def test_clm5_ensemble_members_match_oracle(gpu_lib):
    """The perturbed-parameter ensemble on the CLM5-default step (soil
    resistance, root moisture stress, CanopyFluxes, root sink,
    SoilTemperature, SoilFluxes, the moisture form with the default hydrology)
    with six of the eight parameters acting: medlynslope / medlynintercept per
    patch, om_frac_sf in the soil properties, baseflow_scalar, fff and d_max
    per column.  Every member's result equals the oracle stepped with that
    member's parameters."""
    from ctsm_gb300 import abi, canopy
    from ctsm_gb300.engine import SoilBatch
    nm = 4
    A, npatch, ngrid, rootr, member_col, f = fi.ensemble(nm, seed=12, cols=(200, 500), clm5=True)
    nml = abi.soilwater_movement_nml(1)
    gpu_lib.set_soilwater_movement(nml)
    gpu_lib.set_soilhydrology_params()
    gpu_lib.set_soil_resistance()
    canopy.set_params()
    try:
        hydro, sres = [], []
        for m in range(nm):
            cols = np.nonzero(member_col == m)[0].astype(np.int32) + 1
            hydro.append((cols, abi.SoilHydrologyParams(0.01, 1.0, fi.BASEFLOW_SCALAR * f["baseflow_scalar"][m], 1.0e-5,
                                                        6.0, fi.FFF * f["fff"][m], 0.4, 0.13, 1)))
            sres.append((cols, abi.SoilResistanceParams(1, fi.D_MAX * f["d_max"][m], 0.8)))
        kw = dict(medlyn_per_patch=True, soilfluxes=True, rootmoist=True, swm=nml, soilresis=sres, hydro=hydro)
        R = copy.deepcopy(A)
        full_steps(R, npatch, ngrid, rootr, 2, **kw)
        G = copy.deepcopy(A)
        b = SoilBatch(G, npatch, canopy=True, ngrid=ngrid, per_patch_medlyn=True, soilfluxes=True, rootmoist=True,
                      soilresis=True, hydrology=True, per_column_hydrology=True)
        b.run(2)
        b.sync()
        b.download()
        b.close()
        keys = STATE + ["soilresis", "dsl", "btran", "zwt", "zwt_perched", "fsat", "qflx_infl", "qflx_drain",
                        "qflx_latflow_out", "num_substeps", "eflx_soil_grnd"]
        # qflx_evap_veg = rpp * efpot, efpot a difference of nearly equal
        # humidity terms near saturation (CanopyFluxesMod.F90:1335-1339)
        cancel = CANCEL + ("qflx_drain", "qflx_drain_perched", "eflx_soil_grnd", "qflx_evap_veg")
        spread = noise_spread(lambda B: full_steps(B, npatch, ngrid, rootr, 2, **kw), A, R, fields=cancel,
                              input_ulps=4)
        for k in ("liqcan", "snocan"):
            spread[k] = spread[k] + 1e-9 * (np.abs(A["liqcan"]) + np.abs(A["snocan"]))
        spread["qflx_evap_veg"] = spread["qflx_evap_veg"] + evap_veg_rounding_bound(R)
        errs, bad = compare(G, R, keys, 1e-9, spread)
        assert not bad, {k: errs[k] for k in bad}
        # the three per-column parameters act: members differ where only they differ
        assert len(np.unique(np.round(A["d_max_c"], 12))) == nm
        assert np.ptp(R["soilresis"]) > 0 and (R["zwt"] != A["zwt"]).mean() > 0.5
    finally:
        gpu_lib.set_soilwater_movement(abi.soilwater_movement_nml(0, use_bedrock=0))


def test_plain_clm5_step_matches_oracle(gpu_lib):
    """The CLM5-default step made of drop-in calls alone (ctsm_gb300.plain_step,
    the plain arm of the ensemble benchmark: soil resistance, root moisture
    stress, CanopyFluxes, the root-sink drop-in, SoilTemperature, SoilFluxes,
    SetSoilWaterFractions, the default hydrology around the moisture-form
    SoilWater) against the oracle stepped the same way, one member's
    parameters, 2 steps."""
    from ctsm_gb300 import abi, canopy
    from ctsm_gb300.plain_step import PlainCLM5Step
    A, npatch, ngrid, rootr, member_col, f = fi.ensemble(1, seed=21, cols=(900, 900), clm5=True)
    nml = abi.soilwater_movement_nml(1)
    gpu_lib.set_soilwater_movement(nml)
    try:
        med = (float(f["medlynslope"][0]), float(f["medlynintercept"][0]))
        dmax, bs, fff = (fi.D_MAX * f["d_max"][0], fi.BASEFLOW_SCALAR * f["baseflow_scalar"][0], fi.FFF * f["fff"][0])
        cols = np.arange(1, A["zwt"].shape[0] + 1, dtype=np.int32)
        kw = dict(medlyn_per_patch=True, soilfluxes=True, rootmoist=True, swm=nml,
                  soilresis=[(cols, abi.SoilResistanceParams(1, dmax, 0.8))],
                  hydro=[(cols, abi.SoilHydrologyParams(0.01, 1.0, bs, 1.0e-5, 6.0, fff, 0.4, 0.13, 1))])
        R = copy.deepcopy(A)
        full_steps(R, npatch, ngrid, rootr, 2, **kw)
        G = copy.deepcopy(A)
        st = PlainCLM5Step(G, npatch, ngrid, medlyn=med, d_max=dmax, baseflow_scalar=bs, fff=fff)
        st.step()
        st.step()
        keys = STATE + ["soilresis", "btran", "zwt", "qflx_infl", "qflx_drain", "num_substeps", "eflx_soil_grnd"]
        cancel = CANCEL + ("qflx_drain", "eflx_soil_grnd", "qflx_evap_veg")
        spread = noise_spread(lambda B: full_steps(B, npatch, ngrid, rootr, 2, **kw), A, R, fields=cancel,
                              input_ulps=4)
        for k in ("liqcan", "snocan"):
            spread[k] = spread[k] + 1e-9 * (np.abs(A["liqcan"]) + np.abs(A["snocan"]))
        spread["qflx_evap_veg"] = spread["qflx_evap_veg"] + evap_veg_rounding_bound(R)
        errs, bad = compare(G, R, keys, 1e-9, spread)
        assert not bad, {k: errs[k] for k in bad}
    finally:
        gpu_lib.set_soilwater_movement(abi.soilwater_movement_nml(0, use_bedrock=0))
        gpu_lib.set_soil_resistance()
        gpu_lib.set_soilhydrology_params()
        canopy.set_params()
