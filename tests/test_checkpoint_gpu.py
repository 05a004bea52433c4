"""Checkpoint / restart of a resident batch (the restart role of
restFileMod.F90): a run saved after 3 steps and restored into a fresh batch
continues bit-identically to the uninterrupted run; a file for other sizes
or a truncated file is refused."""
import copy
import os

import numpy as np
import pytest

from ctsm_gb300 import full_inputs as fi
from ctsm_gb300._lib import CtsmError

pytestmark = pytest.mark.gpu
KEYS = ["h2osoi_liq", "h2osoi_ice", "t_soisno", "t_grnd", "h2osoi_vol", "t_veg", "qflx_tran_veg", "zwt", "qcharge",
        "liqcan", "snocan"]


def test_restart_continues_bit_identically(gpu_lib, tmp_path):
    from ctsm_gb300.engine import SoilBatch
    A, npatch, ngrid, rootr = fi.full_state(3000, seed=95)
    ck = os.path.join(tmp_path, "state.ck")
    G = copy.deepcopy(A)
    b = SoilBatch(G, npatch, canopy=True, ngrid=ngrid, rootr=rootr)
    b.run(3)
    b.save(ck)
    b.run(3)
    b.sync()
    b.download()
    b.close()
    H = copy.deepcopy(A)
    b2 = SoilBatch(H, npatch, canopy=True, ngrid=ngrid, rootr=rootr)
    b2.load(ck)
    b2.run(3)
    b2.sync()
    b2.download()
    for k in KEYS:
        np.testing.assert_array_equal(H[k], G[k], err_msg=k)
    # a file of other sizes, and a truncated file, are refused
    S, sp, sg, sr = fi.full_state(100, seed=96)
    b3 = SoilBatch(S, sp, canopy=True, ngrid=sg, rootr=sr)
    with pytest.raises(CtsmError):
        b3.load(ck)
    bad = os.path.join(tmp_path, "cut.ck")
    with open(ck, "rb") as f, open(bad, "wb") as g:
        g.write(f.read()[:4096])
    with pytest.raises(CtsmError):
        b2.load(bad)
    b2.close()
    b3.close()
