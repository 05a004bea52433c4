"""Large drop-in calls over an ascending filter run pipelined (chunks of the
filter copy in, compute and copy out on separate streams); other filters run in
one piece.  Both forms must give bit-identical results, including columns
that are not in the filter (left as they were)."""
import copy

import numpy as np
import pytest

from ctsm_gb300 import abi, inputs, soil

pytestmark = pytest.mark.gpu
DT = 1800.0


def test_pipelined_equals_single_shot(gpu_lib):
    A, npatch = inputs.soil_columns(40000, seed=71, snow=True, nbedrock=(3, 20), forcing="full", npatch_max=3)
    ncol = A["zwt"].shape[0]
    keep = np.arange(1, ncol + 1, dtype=np.int32)
    keep = keep[(keep % 7) != 3]                 # gaps: every 7th column stays out of the filter
    asc = np.ascontiguousarray(keep)
    desc = np.ascontiguousarray(keep[::-1])      # same set, not ascending: one-piece path
    b = abi.Bounds(1, ncol, 1, npatch)
    P, S = copy.deepcopy(A), copy.deepcopy(A)
    soil.SoilWater(b, len(asc), asc, P, DT)
    soil.SoilTemperature(b, len(asc), asc, P, DT)
    soil.SoilWater(b, len(desc), desc, S, DT)
    soil.SoilTemperature(b, len(desc), desc, S, DT)
    out = [n for (n, k, t, u) in abi.SOILWATER_FIELDS + abi.SOILTEMP_FIELDS]
    for k in out:
        np.testing.assert_array_equal(P[k], S[k], err_msg=k)
    skipped = np.setdiff1d(np.arange(ncol), asc - 1)
    for k in ("t_soisno", "h2osoi_liq", "qin", "xmf", "eflx_fgr"):
        np.testing.assert_array_equal(P[k][..., skipped], A[k][..., skipped], err_msg=k)
    assert not np.array_equal(P["t_soisno"], A["t_soisno"])


def _copied(reset=False):
    import ctypes as C
    from ctsm_gb300 import _lib
    L = _lib.load()
    L.ctsmg_copy_bytes.argtypes = [C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_int32]
    h, d = C.c_int64(0), C.c_int64(0)
    _lib.check(L.ctsmg_copy_bytes(C.byref(h), C.byref(d), 1 if reset else 0))
    return h.value, d.value


def test_copy_accounting(gpu_lib):
    """The library counts the bytes each drop-in call moves: the pipelined and
    the one-piece forms move the same bytes for the same work, an ascending
    filter over every column skips the copy-in of the components SoilWater
    overwrites (a filter in another order or with gaps copies them in), and
    a reset zeroes the counters."""
    A, npatch = inputs.soil_columns(40000, seed=72, snow=True, nbedrock=(3, 20))
    ncol = A["zwt"].shape[0]
    b = abi.Bounds(1, ncol, 1, npatch)
    dense = np.arange(1, ncol + 1, dtype=np.int32)
    runs = {}
    for name, f in (("asc", dense), ("desc", np.ascontiguousarray(dense[::-1])),
                    ("gaps", np.ascontiguousarray(dense[(dense % 7) != 3]))):
        S = copy.deepcopy(A)
        _copied(reset=True)
        soil.SoilWater(b, len(f), f, S, DT)
        runs[name] = _copied(reset=True)
    assert _copied() == (0, 0)
    full = sum(A[n].nbytes for (n, k, t, u) in abi.SOILWATER_FIELDS if n in A)
    ngaps = int(np.count_nonzero((dense % 7) != 3))
    # one piece vs pipelined: the same component bytes, except the unfiltered
    # columns between two chunks, which the pipelined form does not move
    per_col = (runs["desc"][0] - 4 * ncol) / ncol
    assert 0 <= (runs["desc"][0] - 4 * ncol) - (runs["gaps"][0] - 4 * ngaps) <= 16 * per_col
    assert 0 < runs["asc"][0] < runs["gaps"][0] <= full + 4 * ncol
    assert 0 < runs["asc"][1] == runs["desc"][1]
    assert 0 <= runs["asc"][1] - runs["gaps"][1] <= 16 * runs["asc"][1] / ncol
