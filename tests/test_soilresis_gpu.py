"""Soil evaporative resistance (calc_soilevap_resis,
SurfaceResistanceMod.F90:190-425) through the drop-in, both methods, against
the oracle; and the resident step computing soilresis before CanopyFluxes."""
import copy
import ctypes as C

import numpy as np
import pytest

from ctsm_gb300 import abi, full_inputs as fi
from tests.parity import compare, noise_spread

pytestmark = pytest.mark.gpu
LS = -abi.NLEVSNO + 1


@pytest.fixture
def soil_sr(gpu_lib):
    yield gpu_lib
    gpu_lib.set_soil_resistance(1, 15.0, 0.8)


def state(ncol, seed):
    A, npatch, ngrid, rootr = fi.full_state(ncol, seed=seed)
    fi.add_soilresis_fields(A)
    r = np.random.Generator(np.random.Philox(seed + 1))
    # dry and saturated top layers beside the drawn ones
    wet = r.choice(ncol, ncol // 10, replace=False)
    A["h2osoi_liq"][1 - LS, wet] = A["watsat"][0, wet] * A["dz"][1 - LS, wet] * 1000.0
    dry = r.choice(ncol, ncol // 10, replace=False)
    A["h2osoi_liq"][1 - LS, dry] = 1e-9
    return A, npatch, ngrid, rootr


def oracle(A, method, d_max, frac, filt, begc=1):
    from oracle import oracle as orc
    ncol = A["zwt"].shape[0]
    io = abi.make_io(abi.SoilResisIO, abi.SOILRESIS_FIELDS, A, ncol)
    f = np.ascontiguousarray(filt, np.int32)
    assert orc.lib().oracle_soilevap_resis(C.byref(abi.Bounds(begc, begc + ncol - 1, 1, 1)), len(f),
                                           f.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(io),
                                           C.byref(abi.SoilResistanceParams(method, d_max, frac))) == 0


@pytest.mark.parametrize("method,d_max,frac", [(1, 15.0, 0.8), (1, 40.0, 0.5), (0, 15.0, 0.8)])
def test_soilevap_resis_matches_oracle(soil_sr, method, d_max, frac):
    A, npatch, ngrid, rootr = state(6000, seed=61)
    filt = np.arange(5, 6001, 2, dtype=np.int32)
    soil_sr.set_soil_resistance(method, d_max, frac)
    G, R = copy.deepcopy(A), copy.deepcopy(A)
    oracle(R, method, d_max, frac, filt)
    soil_sr.calc_soilevap_resis(abi.Bounds(1, 6000, 1, npatch), len(filt), filt, G)
    out = ["dsl", "soilresis"] if method == 1 else ["soilbeta"]
    errs, bad = compare(G, R, out, 1e-12, {})
    assert not bad, {k: errs[k] for k in bad}
    if method == 1:
        d = R["dsl"][filt - 1]
        # wet tops sit at the 0.001 floor of the numerator, dry ones near d_max
        assert d.min() < 0.1 and d.max() > 0.5 * d_max and (R["soilresis"][filt - 1] >= 20.0).all()
    skip = np.setdiff1d(np.arange(6000), filt - 1)
    assert (G[out[0]][skip] == A[out[0]][skip]).all()


def test_resident_step_computes_soilresis(soil_sr):
    """soilresis from the resident soil state at the start of every step,
    then CanopyFluxes, over 3 full steps, against the oracle doing the same."""
    from ctsm_gb300.engine import SoilBatch
    from oracle.steps import full_steps
    A, npatch, ngrid, rootr = state(2500, seed=62)
    R = copy.deepcopy(A)
    filt = np.arange(1, 2501, dtype=np.int32)

    def run(B):
        for _ in range(3):
            oracle(B, 1, 15.0, 0.8, filt)
            full_steps(B, npatch, ngrid, rootr, 1)
    run(R)
    G = copy.deepcopy(A)
    b = SoilBatch(G, npatch, canopy=True, ngrid=ngrid, rootr=rootr, soilresis=True)
    b.run(3)
    b.sync()
    b.download()
    b.close()
    assert (R["soilresis"] != A["soilresis"]).mean() > 0.9
    cancel = ("liqcan", "snocan", "eflx_sh_grnd", "qflx_evap_soi", "xmf")
    spread = noise_spread(run, A, R, fields=cancel, input_ulps=4)
    for k in ("liqcan", "snocan"):
        spread[k] = spread[k] + 1e-9 * (np.abs(A["liqcan"]) + np.abs(A["snocan"]))
    errs, bad = compare(G, R, ["dsl", "soilresis", "t_veg", "t_grnd", "h2osoi_liq", "t_soisno", "qflx_tran_veg"]
                        + list(cancel), 1e-9, spread)
    assert not bad, {k: errs[k] for k in bad}
