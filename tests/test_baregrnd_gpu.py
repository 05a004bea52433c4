"""BareGroundFluxes (BareGroundFluxesMod.F90:73-545) through the drop-in
against the oracle, with both ground-evaporation resistance methods, snow and
surface-water columns, several bare patches per column (the column roughness
takes the last patch's values) and a filter with gaps."""
import copy
import ctypes as C

import numpy as np
import pytest

from ctsm_gb300 import abi, canopy, canopy_inputs, full_inputs as fi
from tests.parity import compare, noise_spread

pytestmark = pytest.mark.gpu
OUT = [n for (n, k, t, u) in abi.BAREGRND_FIELDS if u != "in"]
# flux differences of near-equal humidities / temperatures (dqh, dth, the
# 2 m profile corrections) are compared against the oracle's own spread
CANCEL = ("eflx_sh_grnd", "eflx_sh_tot", "eflx_sh_snow", "eflx_sh_soil", "eflx_sh_h2osfc", "qflx_evap_soi",
          "qflx_evap_tot", "qflx_ev_snow", "qflx_ev_soil", "qflx_ev_h2osfc", "cgrndl", "cgrnd", "q_ref2m",
          "rh_ref2m", "t_ref2m")


@pytest.fixture
def soil_sr(gpu_lib):
    yield gpu_lib
    gpu_lib.set_soil_resistance(1, 15.0, 0.8)


def run_oracle(A, b, filt, ngrid, method):
    from oracle import oracle as orc
    L = orc.lib()
    L.oracle_set_canopy_params(C.byref(canopy_inputs.make_params()), C.byref(canopy_inputs.make_pftcon()), 1, 40)
    ncol = b.endc - b.begc + 1
    npat = b.endp - b.begp + 1
    io = abi.make_io(abi.BareGrndIO, abi.BAREGRND_FIELDS, A, ncol, npat, ngrid, 1)
    f = np.ascontiguousarray(filt, np.int32)
    assert L.oracle_baregroundfluxes(C.byref(b), len(f), f.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(io),
                                     method) == 0


@pytest.mark.parametrize("method", [1, 0])
def test_baregroundfluxes_matches_oracle(soil_sr, method):
    A, npatch, ngrid, rootr = fi.full_state(4000, seed=71)
    fi.add_baregrnd_fields(A, npatch, ngrid)
    canopy.set_params(canopy_inputs.make_params(), canopy_inputs.make_pftcon())
    soil_sr.set_soil_resistance(method, 15.0, 0.8)
    r = np.random.Generator(np.random.Philox(72))
    filt = np.sort(r.choice(np.arange(1, npatch + 1, dtype=np.int32), int(0.8 * npatch), replace=False))
    b = abi.Bounds(1, 4000, 1, npatch)
    G, R = copy.deepcopy(A), copy.deepcopy(A)
    run_oracle(R, b, filt, ngrid, method)
    canopy.BareGroundFluxes(b, len(filt), filt, G, ngrid)
    sp = noise_spread(lambda B: run_oracle(B, b, filt, ngrid, method), A, R, fields=CANCEL, input_ulps=2)
    errs, bad = compare(G, R, OUT, 1e-9, sp)
    assert not bad, {k: errs[k] for k in bad}
    # the column roughness is the last filtered patch's
    pc = A["patch_column"][filt - 1] - 1
    last = {}
    for k, c in enumerate(pc):
        last[c] = filt[k] - 1
    cols = np.array(sorted(last))
    assert (G["z0hg"][cols] == G["z0hg_patch"][[last[c] for c in cols]]).all()
    assert (np.bincount(pc) > 1).any()                   # several bare patches in some columns
    assert (G["num_iter"][filt - 1] == 3).all()
    evap = R["qflx_evap_soi"][filt - 1]
    assert (evap > 0).any() and (evap <= 0).any()
