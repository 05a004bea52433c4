"""A resident batch restored from a restart file in the reference's layout
(SoilBatch.save_restart / load_restart, ctsm_gb300/restart.py) continues the
run bit for bit: a second batch built from the initial inputs and loaded from
the restart written after 3 steps steps to the same state as the original
batch stepping on."""
import copy

import numpy as np
import pytest

from ctsm_gb300 import inputs

pytestmark = pytest.mark.gpu
STATE = ["h2osoi_liq", "h2osoi_ice", "t_soisno", "t_grnd", "t_h2osfc", "h2osoi_vol", "qcharge", "qflx_deficit",
         "xmf", "snow_depth", "int_snow", "h2osno_no_layers", "h2osfc"]


def test_restart_file_continues_the_run(gpu_lib, tmp_path):
    pytest.importorskip("scipy")
    from ctsm_gb300.engine import SoilBatch
    A, npatch = inputs.soil_columns(4096, seed=21, snow=True, nbedrock=(3, 20), forcing="full", npatch_max=3,
                                    h2osfc=True)
    G = copy.deepcopy(A)
    b = SoilBatch(G, npatch)
    b.run(3)
    b.sync()
    written = b.save_restart(tmp_path / "restart.nc")
    assert {"T_SOISNO", "H2OSOI_LIQ", "H2OSOI_ICE", "T_GRND", "SNLSNO"} <= set(written)
    b.run(2)
    b.sync()
    b.download()
    b.close()
    H = copy.deepcopy(A)
    b2 = SoilBatch(H, npatch)
    read = b2.load_restart(tmp_path / "restart.nc")
    assert sorted(read) == sorted(written)
    b2.run(2)
    b2.sync()
    b2.download()
    b2.close()
    for k in STATE:
        assert np.array_equal(G[k], H[k], equal_nan=True), k
