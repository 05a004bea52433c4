"""The allocation-free SoilTemperature entry point against the ordinary one.

ctsmg_soiltemperature_noalloc serves callers that cannot allocate device
memory (their device memory belongs to another runtime, or they must not call
cudaMalloc on this path): they hand over device pointers for every input and
output and the call uses a scratch array built into the library.  This test
puts the inputs on the device itself (with torch, as such a caller's runtime
would), calls the entry point through the C-ABI twice in a row on different
column sets, and checks each result against ctsmg_soiltemperature on the same
inputs.  It lives in the file pytest collects last."""
import copy
import ctypes as C

import numpy as np
import pytest

from ctsm_gb300 import abi, inputs
from tests.parity import compare

pytestmark = pytest.mark.gpu
DT = 1800.0
OUT = [n for (n, k, t, u) in abi.SOILTEMP_FIELDS if u != "in"]
MAX_COLUMNS = 16384


def _bind(L):
    L.ctsmg_soiltemperature_noalloc.argtypes = [C.POINTER(abi.Bounds), C.c_int32, C.c_void_p,
                                                C.POINTER(abi.SoilTempIO), C.c_double, C.c_void_p]
    L.ctsmg_soiltemperature_noalloc.restype = C.c_int32


def _device_io(torch, A, ncol, npatch):
    dev = {k: torch.from_numpy(np.ascontiguousarray(A[k])).cuda() for (k, _, _, _) in abi.SOILTEMP_FIELDS}
    io = abi.SoilTempIO()
    io.ldc, io.ldp = ncol, npatch
    for (k, _, t, _) in abi.SOILTEMP_FIELDS:
        ptype = C.POINTER(C.c_double) if t == abi.F64 else C.POINTER(C.c_int32)
        setattr(io, k, C.cast(C.c_void_p(dev[k].data_ptr()), ptype))
    return dev, io


def _noalloc(torch, L, b, filt, io, n=None):
    """One allocation-free call; filt None passes a NULL filter of n columns."""
    dfilt = None if filt is None else torch.from_numpy(np.ascontiguousarray(filt, dtype=np.int32)).cuda()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    return L.ctsmg_soiltemperature_noalloc(C.byref(b), len(filt) if filt is not None else n,
                                           None if dfilt is None else C.c_void_p(dfilt.data_ptr()), C.byref(io),
                                           DT, C.c_void_p(stream))


def _one_call(torch, soil, L, A, npatch, begc=1, begp=1, filt=None, null_filter=False):
    ncol = A["zwt"].shape[0]
    b = abi.Bounds(begc, begc + ncol - 1, begp, begp + npatch - 1)
    if filt is None:
        filt = np.arange(begc, begc + ncol, dtype=np.int32)
    # ordinary entry point (host buffers)
    R = copy.deepcopy(A)
    soil.SoilTemperature(b, len(filt), filt, R, DT)
    # allocation-free entry point (caller-owned device buffers)
    dev, io = _device_io(torch, A, ncol, npatch)
    rc = _noalloc(torch, L, b, None if null_filter else filt, io, len(filt))
    assert rc == 0, L.ctsmg_last_error().decode()
    G = {k: dev[k].cpu().numpy() for k in OUT}
    errs, bad = compare(G, R, OUT, 1e-9)
    assert not bad, {k: errs[k] for k in bad}


def test_noalloc_matches_dropin_two_calls(gpu_lib):
    torch = pytest.importorskip("torch")
    from ctsm_gb300 import _lib
    L = _lib.load()
    _bind(L)
    A, npatch = inputs.soil_columns(MAX_COLUMNS, seed=41, snow=True, nbedrock=(3, 20), forcing="full",
                                    npatch_max=3, h2osfc=True)
    _one_call(torch, gpu_lib, L, A, npatch)
    # second call in a row: a different, smaller column set with offset bounds
    # and a permuted subset filter, so stale scratch from the first call would show
    B, npb = inputs.soil_columns(5000, seed=42, snow=True, nbedrock=(3, 20), forcing="full", npatch_max=2)
    B["col_patchi"][:] = B["col_patchi"] + 6
    r = np.random.Generator(np.random.Philox(3))
    filt = (r.permutation(5000)[:3100] + 11).astype(np.int32)
    _one_call(torch, gpu_lib, L, B, npb, begc=11, begp=7, filt=filt)


def test_noalloc_rejects_oversize(gpu_lib):
    torch = pytest.importorskip("torch")
    from ctsm_gb300 import _lib
    L = _lib.load()
    _bind(L)
    A, npatch = inputs.soil_columns(64, seed=1)
    dev, io = _device_io(torch, A, 64, npatch)
    b = abi.Bounds(1, MAX_COLUMNS + 1, 1, npatch)
    io.ldc = MAX_COLUMNS + 1
    rc = L.ctsmg_soiltemperature_noalloc(C.byref(b), MAX_COLUMNS + 1, None, C.byref(io), DT, None)
    assert rc == 1  # CTSMG_E_ARG
    assert b"16384" in L.ctsmg_last_error()


def test_noalloc_null_filter_with_offset_bounds(gpu_lib):
    """A NULL filter means columns begc..begc+n-1."""
    torch = pytest.importorskip("torch")
    from ctsm_gb300 import _lib
    L = _lib.load()
    _bind(L)
    A, npatch = inputs.soil_columns(3000, seed=43, snow=True, nbedrock=(3, 20), forcing="full", npatch_max=2)
    A["col_patchi"][:] = A["col_patchi"] + 4
    _one_call(torch, gpu_lib, L, A, npatch, begc=21, begp=5, null_filter=True)


def test_noalloc_rejects_bad_entries_on_the_device_and_recovers(gpu_lib):
    """A filter entry outside begc..endc and a column with nbedrock out of
    range are skipped with CTSMG_E_ARG naming the first bad filter position;
    every other column equals the ordinary call over the good entries, and
    the next good call returns 0 (the device error record is reset)."""
    torch = pytest.importorskip("torch")
    from ctsm_gb300 import _lib
    L = _lib.load()
    _bind(L)
    ncol = 2000
    A, npatch = inputs.soil_columns(ncol, seed=44, snow=True, nbedrock=(3, 20), forcing="full", npatch_max=2)
    b = abi.Bounds(1, ncol, 1, npatch)
    filt = np.arange(1, ncol + 1, dtype=np.int32)
    filt[36] = ncol + 5                      # filter position 37: outside the bounds
    A["nbedrock"][1499] = 0                  # column 1500 (filter position 1500): nbedrock out of range
    good = np.array([f for f in filt if f <= ncol and f != 1500], dtype=np.int32)
    R = copy.deepcopy(A)
    gpu_lib.SoilTemperature(b, len(good), good, R, DT)
    dev, io = _device_io(torch, A, ncol, npatch)
    rc = _noalloc(torch, L, b, filt, io)
    assert rc == 1, rc                                   # CTSMG_E_ARG
    idx, lev = C.c_int32(), C.c_int32()
    L.ctsmg_last_error_index(C.byref(idx), C.byref(lev))
    assert idx.value == 37 and b"filter entry outside" in L.ctsmg_last_error()
    G = {k: dev[k].cpu().numpy() for k in OUT}
    errs, bad = compare(G, R, OUT, 1e-9)
    assert not bad, {k: errs[k] for k in bad}
    # the nbedrock check alone: position 1500
    filt2 = np.arange(1, ncol + 1, dtype=np.int32)
    dev, io = _device_io(torch, A, ncol, npatch)
    assert _noalloc(torch, L, b, filt2, io) == 1
    L.ctsmg_last_error_index(C.byref(idx), C.byref(lev))
    assert idx.value == 1500 and b"nbedrock" in L.ctsmg_last_error()
    # a good call right after: status 0
    A["nbedrock"][1499] = 10
    dev, io = _device_io(torch, A, ncol, npatch)
    assert _noalloc(torch, L, b, filt2, io) == 0, L.ctsmg_last_error()


def test_noalloc_needs_init(gpu_lib):
    """Without ctsmg_init the call refuses to run (CTSMG_E_NOT_INIT), and after
    ctsmg_init it runs again."""
    torch = pytest.importorskip("torch")
    from ctsm_gb300 import _lib
    L = _lib.load()
    _bind(L)
    A, npatch = inputs.soil_columns(256, seed=45, snow=True, nbedrock=(3, 20))
    b = abi.Bounds(1, 256, 1, npatch)
    dev, io = _device_io(torch, A, 256, npatch)
    L.ctsmg_finalize()
    try:
        assert _noalloc(torch, L, b, None, io, 256) == 3     # CTSMG_E_NOT_INIT
    finally:
        gpu_lib.init()
    assert _noalloc(torch, L, b, None, io, 256) == 0, L.ctsmg_last_error()
