"""The water-table and drainage routines around SoilWater (SaturatedExcessRunoff,
PerchedWaterTable, ThetaBasedWaterTable, PerchedLateralFlow,
SubsurfaceLateralFlow) through their drop-in entries, against the oracle:
each alone and in the driver's sequence, on states where their branches act
(frozen layers under a perched table, saturated columns, water tables below
the bedrock, nearly dry layers, an over-full top layer)."""
import copy
import ctypes as C

import numpy as np
import pytest

from ctsm_gb300 import abi, inputs, full_inputs as fi
from tests.parity import compare, noise_spread

pytestmark = pytest.mark.gpu
LS = -abi.NLEVSNO + 1
DT = 1800.0
PAR = dict(aq_sp_yield_min=0.01, n_baseflow=1.0, baseflow_scalar=1.0e-2, perched_baseflow_scalar=1.0e-5, e_ice=6.0,
           fff=0.5, pc=0.4, mu=0.13, h2osfcflag=1)
WHICH = {"SaturatedExcessRunoff": 0, "PerchedWaterTable": 1, "ThetaBasedWaterTable": 2, "PerchedLateralFlow": 3,
         "SubsurfaceLateralFlow": 4, "InfiltrationChain": 5, "WaterTable": 6, "Drainage": 7}
OUT = [n for (n, k, t, u) in abi.HYDROLOGY_FIELDS if u != "in"]


def state(ncol, seed, dry=True):
    A, _ = inputs.soil_columns(ncol, seed=seed, snow=True, nbedrock=(3, 20), zwt=(0.1, 9.5), h2osfc=True)
    r = np.random.Generator(np.random.Philox(seed + 1))
    fi.add_hydrology_fields(A, r)
    soil = slice(1 - LS, abi.NLEVSOI + 1 - LS)
    sat = r.choice(ncol, ncol // 8, replace=False)          # saturated columns
    # (drawn per level: identical saturations in two adjacent layers make the
    # reference's interpolation of the perched table divide by s2 - s1 = 0)
    A["h2osoi_liq"][soil, sat] = r.uniform(0.95, 0.99, (abi.NLEVSOI, len(sat))) * A["watsat"][:abi.NLEVSOI, sat] * \
        A["dz"][soil, sat] * 1000.0
    A["h2osoi_ice"][soil, sat] = 0.0
    dry_cols = r.choice(ncol, ncol // 8, replace=False)     # nearly dry layers
    j = r.integers(1, abi.NLEVSOI + 1, size=len(dry_cols))
    if dry:    # (the moisture form cannot take them: s at its 0.01 floor makes smp ~ 1e25 mm)
        A["h2osoi_liq"][j - LS, dry_cols] = 0.001
    full = r.choice(ncol, ncol // 8, replace=False)         # over-full top layer
    A["h2osoi_liq"][1 - LS, full] = 2.0 * A["watsat"][0, full] * A["dz"][1 - LS, full] * 1000.0
    from ctsm_gb300.inputs import set_soil_water_fractions
    set_soil_water_fractions(A)
    return A


def oracle(A, routines, begc=1, filt=None):
    from oracle import oracle as orc
    ncol = A["zwt"].shape[0]
    f = np.arange(begc, begc + ncol, dtype=np.int32) if filt is None else np.ascontiguousarray(filt, np.int32)
    io = abi.make_io(abi.HydrologyIO, abi.HYDROLOGY_FIELDS, A, ncol)
    P = abi.SoilHydrologyParams(*PAR.values())
    for rt in routines:
        assert orc.lib().oracle_hydrology(C.byref(abi.Bounds(begc, begc + ncol - 1, 1, 1)), len(f),
                                          f.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(io), WHICH[rt],
                                          C.byref(P), DT) == 0


def gpu(soil, A, routines, begc=1, filt=None):
    ncol = A["zwt"].shape[0]
    f = np.arange(begc, begc + ncol, dtype=np.int32) if filt is None else filt
    for rt in routines:
        soil.hydrology(rt, abi.Bounds(begc, begc + ncol - 1, 1, 1), len(f), f, A, DT)


@pytest.mark.parametrize("routine", list(WHICH))
def test_each_routine_matches_oracle(gpu_lib, routine):
    gpu_lib.set_soilhydrology_params(**PAR)
    A = state(5000, seed=81)
    oracle(A, ["PerchedWaterTable"])                  # a consistent frost table / perched table to start from
    G, R = copy.deepcopy(A), copy.deepcopy(A)
    oracle(R, [routine])
    gpu(gpu_lib, G, [routine])
    # the drained water is the flux minus what the layers could not give
    # (drain + tot/dtime): where little was available the difference cancels,
    # so those two fluxes get the oracle's own spread under libm noise
    sp = noise_spread(lambda B: oracle(B, [routine]), A, R, fields=("qflx_drain_perched", "qflx_drain"))
    errs, bad = compare(G, R, OUT, 1e-12, sp)
    assert not bad, {k: errs[k] for k in bad}


def test_driver_sequence_with_filter(gpu_lib):
    """HydrologyNoDrainage's water tables then HydrologyDrainage's lateral
    flows (HydrologyNoDrainageMod.F90:302-372, HydrologyDrainageMod.F90:132-146)
    over a filter with gaps and an offset column range; the branches acted."""
    gpu_lib.set_soilhydrology_params(**PAR)
    A = state(6000, seed=82)
    seq = ["SaturatedExcessRunoff", "InfiltrationChain", "PerchedWaterTable", "ThetaBasedWaterTable",
           "PerchedLateralFlow", "SubsurfaceLateralFlow"]
    r = np.random.Generator(np.random.Philox(83))
    filt = np.sort(r.choice(np.arange(11, 6011, dtype=np.int32), 5000, replace=False))
    G, R = copy.deepcopy(A), copy.deepcopy(A)
    oracle(R, seq, begc=11, filt=filt)
    gpu(gpu_lib, G, seq, begc=11, filt=filt)
    errs, bad = compare(G, R, OUT, 1e-12, {})
    assert not bad, {k: errs[k] for k in bad}
    c = filt - 11
    assert (R["qflx_drain_perched"][c] > 0).any() and (R["qflx_latflow_out"][c] > 0).any()
    assert (R["qflx_latflow_out"][c] == 0).any()          # water table below the bedrock
    assert (R["qflx_ice_runoff_xs"][c] >= 0).all() and (R["qflx_rsub_sat"][c] <= 0).all()
    assert (R["h2osfc"][c] > A["h2osfc"][c]).any()        # top-layer excess went to the surface
    assert (R["qflx_infl_excess"][c] > 0).any() and (R["qflx_h2osfc_drain"][c] > 0).any()
    assert (R["qflx_infl"][c] != 0).all()


def test_resident_steps_with_hydrology(gpu_lib):
    """The moisture form with the default hydrology around it (fsat and the
    infiltration chain feeding SoilWater's qflx_infl before it) in the batched
    engine, 4 steps, per-column baseflow_scalar and fff (two parameter sets
    standing for ensemble members), against the oracle stepped the same way."""
    from ctsm_gb300.engine import SoilBatch
    from oracle.steps import soil_steps
    from tests.parity import noise_spread
    A = state(4000, seed=84, dry=False)
    nml = abi.soilwater_movement_nml(1)
    gpu_lib.set_soilwater_movement(nml)
    gpu_lib.set_soilhydrology_params(**PAR)
    try:
        member = np.arange(4000) % 2
        sets = [dict(PAR, baseflow_scalar=5.0e-3, fff=0.3), dict(PAR, baseflow_scalar=2.0e-2, fff=0.8)]
        A["baseflow_scalar_c"] = np.array([sets[m]["baseflow_scalar"] for m in member])
        A["fff_c"] = np.array([sets[m]["fff"] for m in member])
        hydro = [(np.nonzero(member == m)[0].astype(np.int32) + 1, abi.SoilHydrologyParams(*sets[m].values()))
                 for m in (0, 1)]
        npatch = A["wtcol"].shape[0]
        R = copy.deepcopy(A)
        soil_steps(R, npatch, 4, swm=nml, hydro=hydro)
        G = copy.deepcopy(A)
        b = SoilBatch(G, npatch, dtime=DT, hydrology=True, per_column_hydrology=True)
        b.run(4)
        b.sync()
        b.download()
        b.close()
        keys = ["h2osoi_liq", "h2osoi_ice", "t_soisno", "zwt", "zwt_perched", "frost_table", "h2osfc", "fsat", "qflx_infl",
                "qflx_drain", "qflx_drain_perched", "qflx_latflow_out", "num_substeps", "h2osoi_vol"]
        spread = noise_spread(lambda B: soil_steps(B, npatch, 4, swm=nml, hydro=hydro), A, R,
                              fields=("qflx_drain", "qflx_drain_perched", "xmf"))
        errs, bad = compare(G, R, keys, 1e-9, spread)
        assert not bad, {k: errs[k] for k in bad}
        assert (R["zwt"] != A["zwt"]).mean() > 0.5          # the water table is prognostic
    finally:
        gpu_lib.set_soilwater_movement(abi.soilwater_movement_nml(0, use_bedrock=0))


def test_aquifer_path_sequence(gpu_lib):
    """The aquifer-layer path after the Zeng-Decker SoilWater: WaterTable then
    Drainage (HydrologyNoDrainageMod.F90:356-359, HydrologyDrainageMod.F90:132-137)
    over water tables above, inside and below the soil column, with recharge
    of both signs and perched water over frozen layers."""
    gpu_lib.set_soilhydrology_params(**PAR)
    A = state(6000, seed=85)
    r = np.random.Generator(np.random.Philox(86))
    A["qcharge"] = r.uniform(-2e-4, 2e-4, 6000)
    seq = ["WaterTable", "Drainage"]
    G, R = copy.deepcopy(A), copy.deepcopy(A)
    oracle(R, seq)
    gpu(gpu_lib, G, seq)
    errs, bad = compare(G, R, OUT, 1e-12, {})
    assert not bad, {k: errs[k] for k in bad}
    deep = A["zwt"] > 8.6
    assert deep.any() and (R["wa"][deep] != A["wa"][deep]).any()
    assert (R["qflx_drain_perched"] > 0).any() and (R["qflx_drain"] > 0).any()


def test_resident_zd09_steps_with_aquifer_hydrology(gpu_lib):
    """The Zeng-Decker SoilWater with the aquifer-layer hydrology around it
    (fsat and the infiltration chain before it, WaterTable and Drainage after
    it) in the batched engine, 4 steps, two fff sets, against the oracle."""
    from ctsm_gb300.engine import SoilBatch
    from oracle.steps import soil_steps
    A = state(4000, seed=87)
    gpu_lib.set_soilhydrology_params(**PAR)
    member = np.arange(4000) % 2
    sets = [dict(PAR, fff=0.3), dict(PAR, fff=0.8)]
    A["baseflow_scalar_c"] = np.array([sets[m]["baseflow_scalar"] for m in member])
    A["fff_c"] = np.array([sets[m]["fff"] for m in member])
    hydro = [(np.nonzero(member == m)[0].astype(np.int32) + 1, abi.SoilHydrologyParams(*sets[m].values()))
             for m in (0, 1)]
    npatch = A["wtcol"].shape[0]
    R = copy.deepcopy(A)
    soil_steps(R, npatch, 4, hydro=hydro)
    G = copy.deepcopy(A)
    b = SoilBatch(G, npatch, dtime=DT, hydrology=True, per_column_hydrology=True)
    b.run(4)
    b.sync()
    b.download()
    b.close()
    keys = ["h2osoi_liq", "h2osoi_ice", "t_soisno", "zwt", "zwt_perched", "frost_table", "h2osfc", "fsat", "qflx_infl",
            "wa", "h2osoi_vol", "qcharge"]
    # layers drained down to watmin keep liq = liq + layer with layer ~ -(liq - watmin):
    # their few remaining kg/m2 carry the rounding of the whole layer, so the
    # liquid gets the oracle's own spread as well
    spread = noise_spread(lambda B: soil_steps(B, npatch, 4, hydro=hydro), A, R,
                          fields=("qflx_drain", "qflx_drain_perched", "xmf", "qcharge", "h2osoi_liq", "h2osoi_vol"))
    errs, bad = compare(G, R, keys + ["qflx_drain", "qflx_drain_perched"], 1e-9, spread)
    assert not bad, {k: errs[k] for k in bad}
    assert (R["zwt"] != A["zwt"]).mean() > 0.5 and (R["wa"] != A["wa"]).any()

