"""Parity of the CUDA SoilWater / SoilTemperature drop-in calls with the oracle
(one 1800 s step, FP64, relative error <= 1e-9 on every written component)."""
import copy
import ctypes as C

import numpy as np
import pytest

from ctsm_gb300 import abi, inputs
from oracle import oracle as orc
from tests.parity import compare, noise_spread, fgr_rounding_bound

pytestmark = pytest.mark.gpu
DT = 1800.0
TOL = 1e-9

SW_OUT = [n for (n, k, t, u) in abi.SOILWATER_FIELDS if u != "in"]
ST_OUT = [n for (n, k, t, u) in abi.SOILTEMP_FIELDS if u != "in"]


def run_oracle(A, npatch, filt, begc=1, begp=1, which=("water", "temp"), snow_method=0):
    L = orc.lib()
    ncol = A["zwt"].shape[0]
    b = abi.Bounds(begc, begc + ncol - 1, begp, begp + npatch - 1)
    f = np.ascontiguousarray(filt, np.int32)
    fp = f.ctypes.data_as(C.POINTER(C.c_int32))
    if "water" in which:
        io = abi.make_io(abi.SoilWaterIO, abi.SOILWATER_FIELDS, A, ncol)
        assert L.oracle_soilwater(C.byref(b), len(f), fp, C.byref(io), 6.0, DT) == 0
    if "temp" in which:
        io = abi.make_io(abi.SoilTempIO, abi.SOILTEMP_FIELDS, A, ncol, npatch)
        assert L.oracle_soiltemperature(C.byref(b), len(f), fp, C.byref(io), DT, snow_method) == 0


def run_gpu(soil, A, npatch, filt, begc=1, begp=1, which=("water", "temp")):
    ncol = A["zwt"].shape[0]
    b = abi.Bounds(begc, begc + ncol - 1, begp, begp + npatch - 1)
    if "water" in which:
        soil.SoilWater(b, len(filt), filt, A, DT)
    if "temp" in which:
        soil.SoilTemperature(b, len(filt), filt, A, DT)


def check_case(soil, A, npatch, filt=None, begc=1, begp=1, which=("water", "temp")):
    ncol = A["zwt"].shape[0]
    if filt is None:
        filt = np.arange(begc, begc + ncol, dtype=np.int32)
    G = copy.deepcopy(A)
    R = copy.deepcopy(A)
    run_oracle(R, npatch, filt, begc, begp, which)
    run_gpu(soil, G, npatch, filt, begc, begp, which)
    fields = (SW_OUT if "water" in which else []) + (ST_OUT if "temp" in which else [])
    spread = oracle_spread(A, R, npatch, filt, begc, begp, which)
    errs, bad = compare(G, R, sorted(set(fields)), TOL, spread)
    assert not bad, {k: errs[k] for k in bad}
    return errs


def oracle_spread(A, R, npatch, filt, begc, begp, which, snow_method=0):
    """Acceptance band of the cancellation diagnostics: the oracle's spread
    under libm noise, plus for eflx_fgr the rounding bound of the temperatures
    it differences."""
    sp = noise_spread(lambda B: run_oracle(B, npatch, filt, begc, begp, which, snow_method), A, R)
    if "temp" in which:
        sp["eflx_fgr"] = sp["eflx_fgr"] + fgr_rounding_bound(R)
    return sp


def test_plain_small_config(gpu_lib):
    """4,096 columns, no snow, nbedrock = 20, the ground-flux forcing rule."""
    A, npatch = inputs.soil_columns(4096, seed=0)
    check_case(gpu_lib, A, npatch)


def test_uneven_columns_full_forcing(gpu_lib):
    """snl 0..-12, nbedrock 3..20, 1-4 patches, every flux drawn, standing water."""
    A, npatch = inputs.soil_columns(8192, seed=11, snow=True, nbedrock=(3, 20), forcing="full",
                                    npatch_max=4, h2osfc=True)
    check_case(gpu_lib, A, npatch)


@pytest.mark.parametrize("ncol", [1, 31, 33, 65, 129])
def test_ragged_sizes(gpu_lib, ncol):
    A, npatch = inputs.soil_columns(ncol, seed=100 + ncol, snow=True, nbedrock=(3, 20), forcing="full",
                                    npatch_max=3)
    check_case(gpu_lib, A, npatch)


@pytest.mark.parametrize("snl", list(range(-12, 1)))
def test_each_snow_depth(gpu_lib, snl):
    A, npatch = inputs.soil_columns(256, seed=500 - snl, snow=True, nbedrock=(3, 20), forcing="full")
    A["snl"][:] = snl
    # rebuild a consistent snow geometry for the forced snl
    r = np.random.Generator(np.random.Philox(9000 - snl))
    LS = -abi.NLEVSNO + 1
    A["zi"][abi.NLEVSNO] = 0.0
    for j in range(0, LS - 1, -1):
        row = j - LS
        act = j >= snl + 1
        dzj = r.uniform(0.01, 0.5, 256) if act else np.zeros(256)
        A["dz"][row] = dzj
        zij = A["zi"][j + abi.NLEVSNO]
        A["zi"][j - 1 + abi.NLEVSNO] = zij - dzj if act else 0.0
        A["z"][row] = zij - 0.5 * dzj if act else 0.0
        tot = r.uniform(50, 400, 256) * dzj
        A["h2osoi_liq"][row] = 0.05 * tot
        A["h2osoi_ice"][row] = 0.95 * tot
        A["t_soisno"][row] = r.uniform(230.0, 273.15, 256) if act else 0.0
    A["frac_sno_eff"][:] = 1.0 if snl < 0 else 0.0
    A["sabg_lyr"][:] = 0.0
    A["sabg_lyr"][snl + 1 - LS] = A["sabg"]
    check_case(gpu_lib, A, npatch)


def test_deep_water_table(gpu_lib):
    """zwt below the soil column (jwt == nlevsoi branch, aquifer node active)."""
    A, npatch = inputs.soil_columns(2048, seed=7, zwt=(8.7, 14.0), snow=True)
    check_case(gpu_lib, A, npatch, which=("water",))
    A, npatch = inputs.soil_columns(2048, seed=8, zwt=(0.0, 0.015))  # zwt in the top layer (jwt = 0)
    check_case(gpu_lib, A, npatch, which=("water",))


def test_filter_subset_and_offset_bounds(gpu_lib):
    """A permuted subset filter, begc != 1: untouched columns must stay as input."""
    A, npatch = inputs.soil_columns(3000, seed=21, snow=True, nbedrock=(3, 20), forcing="full", npatch_max=2)
    begc, begp = 101, 51
    A["col_patchi"][:] = A["col_patchi"] + (begp - 1)
    r = np.random.Generator(np.random.Philox(5))
    filt = (r.permutation(3000)[:1700] + begc).astype(np.int32)
    before = copy.deepcopy(A)
    check_case(gpu_lib, A, npatch, filt=filt, begc=begc, begp=begp)
    G = copy.deepcopy(A)
    run_gpu(gpu_lib, G, npatch, filt, begc, begp)
    untouched = np.setdiff1d(np.arange(3000), filt - begc)
    for k in ("h2osoi_liq", "t_soisno", "qcharge", "t_grnd"):
        np.testing.assert_array_equal(G[k][..., untouched], before[k][..., untouched])


def test_sturm_snow_conductivity(gpu_lib):
    from ctsm_gb300 import soil
    soil.init(snow_thermal_cond_method=1)
    try:
        A, npatch = inputs.soil_columns(1024, seed=33, snow=True, nbedrock=(3, 20))
        G = copy.deepcopy(A)
        R = copy.deepcopy(A)
        filt = np.arange(1, 1025, dtype=np.int32)
        run_oracle(R, npatch, filt, which=("temp",), snow_method=1)
        run_gpu(soil, G, npatch, filt, which=("temp",))
        spread = oracle_spread(A, R, npatch, filt, 1, 1, ("temp",), snow_method=1)
        errs, bad = compare(G, R, ST_OUT, TOL, spread)
        assert not bad, {k: errs[k] for k in bad}
    finally:
        soil.init(snow_thermal_cond_method=0)
