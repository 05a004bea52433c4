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


def _one_call(torch, soil, L, A, npatch, begc=1, begp=1, filt=None):
    ncol = A["zwt"].shape[0]
    b = abi.Bounds(begc, begc + ncol - 1, begp, begp + npatch - 1)
    if filt is None:
        filt = np.arange(begc, begc + ncol, dtype=np.int32)
    # ordinary entry point (host buffers)
    R = copy.deepcopy(A)
    soil.SoilTemperature(b, len(filt), filt, R, DT)
    # allocation-free entry point (caller-owned device buffers)
    dev, io = _device_io(torch, A, ncol, npatch)
    dfilt = torch.from_numpy(filt.copy()).cuda()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.ctsmg_soiltemperature_noalloc(C.byref(b), len(filt), C.c_void_p(dfilt.data_ptr()), C.byref(io), DT,
                                          C.c_void_p(stream))
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
