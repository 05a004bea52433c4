"""SoilWater's moisture form (soilwater_movement_method = 1,
SoilWaterMovementMod.F90:976-2160) and the use_flexibleCN fix (:331-368)
through the ctsmg_soilwater drop-in, against the oracle: one 1800 s step,
FP64, relative error <= 1e-9, the adaptive sub-step counts identical."""
import copy
import ctypes as C

import numpy as np
import pytest

from ctsm_gb300 import abi, inputs
from oracle import oracle as orc
from tests.parity import compare, noise_spread

pytestmark = pytest.mark.gpu
DT = 1800.0
LS = -abi.NLEVSNO + 1
FIELDS = abi.SOILWATER_FIELDS + abi.SOILWATER_EXTRA
MF_OUT = ["h2osoi_liq", "qcharge", "qin", "qout", "smp_l", "hk_l", "num_substeps"]
CANCEL = ("qin", "qout", "qcharge")


@pytest.fixture
def soil_mf(gpu_lib):
    yield gpu_lib
    gpu_lib.set_soilwater_movement(abi.soilwater_movement_nml(0, use_bedrock=0))


def run_oracle(A, filt, nml, begc=1):
    L = orc.lib()
    ncol = A["zwt"].shape[0]
    b = abi.Bounds(begc, begc + ncol - 1, 1, 1)
    f = np.ascontiguousarray(filt, np.int32)
    fp = f.ctypes.data_as(C.POINTER(C.c_int32))
    io = abi.make_io(abi.SoilWaterIO, FIELDS, A, ncol)
    if nml.soilwater_movement_method == 1:
        e = C.c_int(0)
        assert L.oracle_soilwater_mf(C.byref(b), len(f), fp, C.byref(io), 6.0, DT, C.byref(nml), C.byref(e)) == 0
    else:
        assert L.oracle_soilwater(C.byref(b), len(f), fp, C.byref(io), 6.0, DT) == 0
    if nml.use_flexibleCN:
        L.oracle_flexcn_fix(C.byref(b), len(f), fp, C.byref(io))


def check(soil, A, nml, filt=None, begc=1, extra=()):
    ncol = A["zwt"].shape[0]
    if filt is None:
        filt = np.arange(begc, begc + ncol, dtype=np.int32)
    soil.set_soilwater_movement(nml)
    G, R = copy.deepcopy(A), copy.deepcopy(A)
    run_oracle(R, filt, nml, begc)
    soil.SoilWater(abi.Bounds(begc, begc + ncol - 1, 1, 1), len(filt), filt, G, DT)
    out = (MF_OUT if nml.soilwater_movement_method == 1 else
           [n for (n, k, t, u) in abi.SOILWATER_FIELDS if u != "in"]) + list(extra)
    sp = noise_spread(lambda B: run_oracle(B, filt, nml, begc), A, R,
                      fields=tuple(k for k in CANCEL if k in out))
    errs, bad = compare(G, R, out, 1e-9, sp)
    assert not bad, {k: errs[k] for k in bad}
    if nml.soilwater_movement_method == 1:
        cols = filt - begc
        assert (G["num_substeps"][cols] == R["num_substeps"][cols]).all()
        assert (R["num_substeps"][cols] >= 1).all()
    return G, R


def soil_state(ncol, seed, nbedrock=(3, 20), zwt=(0.5, 8.0)):
    A, _ = inputs.soil_columns(ncol, seed=seed, snow=True, nbedrock=nbedrock, zwt=zwt, forcing="full")
    r = np.random.Generator(np.random.Philox(seed + 100))
    A["qflx_rootsoi"][:] = r.uniform(0.0, 2e-5, A["qflx_rootsoi"].shape)
    A["qflx_infl"][:] = r.uniform(0.0, 5e-4, ncol)
    return A


def test_zero_flux_bedrock(soil_mf):
    """The CLM5 default: bc_zero_flux at nbedrock (3..20 layers), inexpensive
    error estimate; both sub-step rules (halving and doubling) act."""
    A = soil_state(6000, seed=21)
    G, R = check(soil_mf, A, abi.soilwater_movement_nml(1))
    n = R["num_substeps"]
    assert (n == 1).any() and (n > 5).any()


def test_free_drainage_and_expensive_estimate(soil_mf):
    A = soil_state(3000, seed=22, nbedrock=(20, 20))
    check(soil_mf, A, abi.soilwater_movement_nml(1, lower=1, use_bedrock=0))
    A = soil_state(3000, seed=23)
    check(soil_mf, A, abi.soilwater_movement_nml(1, flux_calculation=42))


def test_water_table_boundary(soil_mf):
    """bc_waterTable with the water table inside and below the column
    (zi(nlevsoi) = 8.6 m), compute_qcharge on the last trial's state."""
    A = soil_state(4000, seed=24, nbedrock=(20, 20), zwt=(0.5, 9.5))
    G, R = check(soil_mf, A, abi.soilwater_movement_nml(1, lower=3, use_bedrock=0))
    assert (A["zwt"] > 8.6).any() and (R["qcharge"] != 0).any()


def test_filter_subset_and_offset(soil_mf):
    A = soil_state(3000, seed=25)
    r = np.random.Generator(np.random.Philox(26))
    filt = np.sort(r.choice(np.arange(101, 3101, dtype=np.int32), 2000, replace=False))
    G, R = check(soil_mf, A, abi.soilwater_movement_nml(1), filt=filt, begc=101)
    skip = np.setdiff1d(np.arange(3000), filt - 101)
    assert (G["h2osoi_liq"][:, skip] == A["h2osoi_liq"][:, skip]).all()


@pytest.mark.parametrize("method", [0, 1])
def test_flexible_cn_fix(soil_mf, method):
    """Negative liquid is borrowed from the layer underneath, the bottom
    layer is topped up from the aquifer (wa) and h2osoi_vol is refreshed.
    ZD09: negative liquid planted in the input, which it carries through.
    Moisture form: a strong root sink in the top layers drives the solve's
    own result negative (negative input liquid puts s at its 0.01 floor, where
    smp ~ s^-b exceeds 1e25 mm and the reference's dgtsv meets a zero pivot)."""
    A = soil_state(3000, seed=27 + method, nbedrock=(20, 20) if method == 0 else (3, 20))
    r = np.random.Generator(np.random.Philox(29))
    cols = r.choice(3000, 300, replace=False)
    for c in cols:
        if method == 0:
            j = int(r.integers(1, abi.NLEVSOI + 1))
            A["h2osoi_liq"][j - LS, c] = -r.uniform(0.0, 0.5)
        else:
            A["qflx_rootsoi"][int(r.integers(0, 3)), c] = 3e-3
    nml = abi.soilwater_movement_nml(method, use_flexibleCN=1, use_bedrock=1 if method == 1 else 0)
    if method == 1:            # the fix has something to do
        B = copy.deepcopy(A)
        run_oracle(B, np.arange(1, 3001, dtype=np.int32), abi.soilwater_movement_nml(1))
        assert (B["h2osoi_liq"][1 - LS:abi.NLEVSOI + 1 - LS] < 0).any()
    G, R = check(soil_mf, A, nml, extra=["wa", "h2osoi_vol"])
    top = slice(1 - LS, abi.NLEVSOI - LS)          # levels 1 .. nlevsoi-1 end non-negative
    assert (R["h2osoi_liq"][top] >= 0).all() and (G["h2osoi_liq"][top] >= 0).all()
    if method == 0:
        assert (R["wa"] != A["wa"]).any()


STATE = ["h2osoi_liq", "h2osoi_ice", "t_soisno", "t_grnd", "h2osoi_vol", "qcharge", "xmf", "num_substeps",
         "icefrac", "eff_porosity"]


@pytest.mark.parametrize("lower,nbedrock", [(2, (3, 20)), (3, (20, 20))])
def test_resident_steps_with_moisture_form(soil_mf, lower, nbedrock):
    """The batched engine's order 0 (SoilWater then SoilTemperature) with the
    moisture form in its own kernel, 4 steps, against the oracle stepped the
    same way; column water closes with the zero-flux boundary."""
    from ctsm_gb300.engine import SoilBatch
    from oracle.steps import soil_steps
    A, npatch = inputs.soil_columns(4000, seed=31, snow=True, nbedrock=nbedrock, forcing="full", npatch_max=3,
                                    zwt=(0.5, 9.5))
    r = np.random.Generator(np.random.Philox(32))
    A["qflx_rootsoi"][:] = r.uniform(0.0, 2e-5, A["qflx_rootsoi"].shape)
    nml = abi.soilwater_movement_nml(1, lower=lower, use_bedrock=1 if lower == 2 else 0)
    soil_mf.set_soilwater_movement(nml)
    R = copy.deepcopy(A)
    soil_steps(R, npatch, 4, swm=nml)
    G = copy.deepcopy(A)
    b = SoilBatch(G, npatch, dtime=DT, balance=lower == 2, skip_steps=0)
    b.run(4)
    b.sync()
    b.download()
    bal = b.balance() if lower == 2 else None
    b.close()
    spread = noise_spread(lambda B: soil_steps(B, npatch, 4, swm=nml), A, R, fields=("xmf", "qcharge"))
    errs, bad = compare(G, R, STATE, 1e-9, spread)
    assert not bad, {k: errs[k] for k in bad}
    assert (G["num_substeps"] == R["num_substeps"]).all()
    if bal is not None:
        assert np.abs(bal[0]).max() < 1e-8          # errh2o (mm) over the 4 steps


def test_full_step_with_moisture_form(soil_mf):
    """Driver order with SoilFluxes and the moisture form after the heat solve
    (clm_driver.F90:900, 921, 950), 3 steps."""
    from ctsm_gb300 import full_inputs as fi
    from ctsm_gb300.engine import SoilBatch
    from oracle.steps import full_steps
    A, npatch, ngrid, rootr = fi.full_state(2500, seed=37)
    fi.add_soilfluxes_fields(A, npatch, ngrid)
    nml = abi.soilwater_movement_nml(1)
    soil_mf.set_soilwater_movement(nml)
    R = copy.deepcopy(A)
    full_steps(R, npatch, ngrid, rootr, 3, soilfluxes=True, swm=nml)
    G = copy.deepcopy(A)
    b = SoilBatch(G, npatch, canopy=True, ngrid=ngrid, rootr=rootr, soilfluxes=True)
    b.run(3)
    b.sync()
    b.download()
    b.close()
    cancel = ("liqcan", "snocan", "eflx_sh_grnd", "qflx_evap_soi", "xmf", "eflx_soil_grnd", "qcharge")
    spread = noise_spread(lambda B: full_steps(B, npatch, ngrid, rootr, 3, soilfluxes=True, swm=nml), A, R,
                          fields=cancel, input_ulps=4)
    for k in ("liqcan", "snocan"):
        spread[k] = spread[k] + 1e-9 * (np.abs(A["liqcan"]) + np.abs(A["snocan"]))
    errs, bad = compare(G, R, ["h2osoi_liq", "h2osoi_ice", "t_soisno", "t_grnd", "h2osoi_vol", "t_veg",
                               "qflx_tran_veg", "num_substeps", "eflx_soil_grnd"] + list(cancel), 1e-9, spread)
    assert not bad, {k: errs[k] for k in bad}


def test_mf_work_orders_give_identical_bits(soil_mf):
    """The persistent sub-step kernel's bucketed work order (previous step's
    sub-step count, bedrock depth) changes which lane takes which column and
    when, never a column's arithmetic: 4 steps in the bucketed order, in
    position order and after the autotuner (which times both) give the same
    bits, and the tuner reports both work orders."""
    from ctsm_gb300.engine import SoilBatch
    A, npatch = inputs.soil_columns(9000, seed=41, snow=True, nbedrock=(3, 20), forcing="full", npatch_max=3,
                                    zwt=(0.5, 9.5))
    r = np.random.Generator(np.random.Philox(42))
    A["qflx_rootsoi"][:] = r.uniform(0.0, 2e-5, A["qflx_rootsoi"].shape)
    A["qflx_infl"][:] = r.uniform(0.0, 5e-4, A["zwt"].shape[0])
    soil_mf.set_soilwater_movement(abi.soilwater_movement_nml(1))
    out = []
    for mode in ("sorted", "positions", "tuned"):
        G = copy.deepcopy(A)
        b = SoilBatch(G, npatch, dtime=DT)
        if mode != "tuned":
            b.set_mf_order(mode == "sorted")
        b.run(2)
        if mode == "tuned":
            t = b.tune(trial_steps=1)
            assert t["mf_order"] in ("sub-steps,bedrock", "positions")
            # a soil-only batch tunes its column order too: 4 orders x 2 work orders
            assert len(t["ms_per_step"]) == 8 and all(len(v) == 3 for v in t["ms_per_step"].values())
            assert sum(k.endswith("/positions") for k in t["ms_per_step"]) == 4
        b.run(2)
        b.sync()
        b.download()
        b.close()
        out.append(G)
    assert (out[0]["num_substeps"] >= 1).all() and out[0]["num_substeps"].max() > 1
    for G in out[1:]:
        for k in STATE + ["qin", "qout", "smp_l", "hk_l"]:
            assert np.array_equal(G[k], out[0][k], equal_nan=True), k
