"""The pipelined drop-in calls' two copy-in paths: with page-locked host
arrays a gather kernel reads each chunk's column slices through the arrays'
device-mapped addresses; with ordinary (pageable) arrays, or copy mode 1, the
copy engines move them.  SoilWater + SoilTemperature over 40,000 columns (a
pipelined call) give the same bits on every path, the per-chunk timeline
reports the chunks, and the library's byte counts agree between the paths."""
import copy
import ctypes as C

import numpy as np
import pytest

from ctsm_gb300 import abi, inputs

pytestmark = pytest.mark.gpu
DT = 1800.0


def _pinned(A):
    import torch
    H = {}
    for k, v in A.items():
        t = torch.empty(v.shape, dtype=torch.float64 if v.dtype == np.float64 else torch.int32).pin_memory()
        h = t.numpy()
        h[...] = v
        H[k] = h
    return H


def _pair(soil, S, ncol, npatch):
    bnd = abi.Bounds(1, ncol, 1, npatch)
    filt = np.arange(1, ncol + 1, dtype=np.int32)
    soil.SoilWater(bnd, ncol, filt, S, DT)
    soil.SoilTemperature(bnd, ncol, filt, S, DT)


def test_gather_and_engine_copies_give_the_same_bits(gpu_lib):
    from ctsm_gb300 import _lib
    L = _lib.load()
    L.ctsmg_set_copy_mode.argtypes = [C.c_int32]
    L.ctsmg_copy_bytes.argtypes = [C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_int32]
    L.ctsmg_pipe_trace.argtypes = [C.c_int32, C.POINTER(C.c_float), C.c_int32, C.POINTER(C.c_int32)]
    A, npatch = inputs.soil_columns(40000, seed=91, snow=True, nbedrock=(3, 20), forcing="full", npatch_max=3)
    ncol = A["zwt"].shape[0]
    runs = {}
    h2d = {}
    try:
        for name, mode, pinned in (("gather", 0, True), ("engines", 1, True), ("pageable", 0, False)):
            _lib.check(L.ctsmg_set_copy_mode(mode))
            S = _pinned(A) if pinned else copy.deepcopy(A)
            bi, bo = C.c_int64(), C.c_int64()
            _lib.check(L.ctsmg_copy_bytes(C.byref(bi), C.byref(bo), 1))
            _lib.check(L.ctsmg_pipe_trace(1, None, 0, None))
            _pair(gpu_lib, S, ncol, npatch)
            buf = (C.c_float * (7 * 64))()
            n = C.c_int32()
            _lib.check(L.ctsmg_pipe_trace(0, buf, 64, C.byref(n)))
            assert n.value > 1                           # the SoilTemperature call ran in chunks
            marks = np.array(buf[:7 * n.value]).reshape(n.value, 7)
            assert (marks[:, 1] >= marks[:, 0]).all() and (marks[:, 3] >= marks[:, 2]).all()
            assert (marks[:, 2] >= marks[:, 1] - 1e-3).all()      # a chunk's kernel starts after its copy-in
            _lib.check(L.ctsmg_copy_bytes(C.byref(bi), C.byref(bo), 1))
            h2d[name] = bi.value
            runs[name] = {k: np.array(v) for k, v in S.items()}
    finally:
        L.ctsmg_set_copy_mode(0)
    assert h2d["gather"] == h2d["engines"] == h2d["pageable"]
    for name in ("engines", "pageable"):
        for k in runs["gather"]:
            assert np.array_equal(runs["gather"][k], runs[name][k], equal_nan=True), (name, k)
    assert not np.array_equal(runs["gather"]["t_soisno"], A["t_soisno"])   # the calls did work


def test_copy_mode_rejects_unknown_modes(gpu_lib):
    from ctsm_gb300 import _lib
    L = _lib.load()
    L.ctsmg_set_copy_mode.argtypes = [C.c_int32]
    assert L.ctsmg_set_copy_mode(2) != 0
    assert L.ctsmg_set_copy_mode(0) == 0


def test_time_constant_inputs_kept_between_calls(gpu_lib):
    """ctsmg_set_time_constant_inputs(1): the pipelined calls keep their device
    copies of the soil properties and the soil-layer geometry between calls.
    Two pairs of calls give the same bits as with every input copied, the
    second pair copies fewer bytes in, and after a soil property changes on
    the host and ctsmg_invalidate_time_constant_inputs() the next pair sees
    the new values."""
    from ctsm_gb300 import _lib
    L = _lib.load()
    L.ctsmg_set_time_constant_inputs.argtypes = [C.c_int32]
    L.ctsmg_copy_bytes.argtypes = [C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_int32]
    A, npatch = inputs.soil_columns(40000, seed=93, snow=True, nbedrock=(3, 20), forcing="full", npatch_max=3)
    ncol = A["zwt"].shape[0]

    def h2d():
        bi, bo = C.c_int64(), C.c_int64()
        _lib.check(L.ctsmg_copy_bytes(C.byref(bi), C.byref(bo), 1))
        return bi.value

    def run(resident, change=False):
        _lib.check(L.ctsmg_set_time_constant_inputs(1 if resident else 0))
        S = copy.deepcopy(A)
        h2d()
        _pair(gpu_lib, S, ncol, npatch)
        first = h2d()
        _pair(gpu_lib, S, ncol, npatch)
        second = h2d()
        if change:
            S["watsat"][...] = S["watsat"] * 1.01          # a soil property edited on the host
            L.ctsmg_invalidate_time_constant_inputs()
            _pair(gpu_lib, S, ncol, npatch)
        return S, first, second

    try:
        S0, f0, s0 = run(False)
        S1, f1, s1 = run(True)
        C0, _, _ = run(False, change=True)
        C1, _, _ = run(True, change=True)
    finally:
        L.ctsmg_set_time_constant_inputs(0)
    assert f1 == f0 == s0 and s1 < s0
    for k in A:
        assert np.array_equal(S1[k], S0[k], equal_nan=True), k
        assert np.array_equal(C1[k], C0[k], equal_nan=True), k
    assert not np.array_equal(C0["h2osoi_liq"], S0["h2osoi_liq"])
