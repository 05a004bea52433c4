"""Python handle on the batched resident mode of libctsm_gpu.so."""
import ctypes as C

import numpy as np

from . import abi
from ._lib import load, check


def _bind(L):
    if getattr(L, "_batch_bound", False):
        return
    P = C.POINTER
    L.ctsmg_batch_create.argtypes = [P(C.c_void_p), P(abi.SoilWaterIO), P(abi.SoilTempIO), C.c_int32, C.c_int32,
                                     C.c_double, C.c_double, C.c_int32]
    L.ctsmg_batch_run.argtypes = [C.c_void_p, C.c_int32, P(C.c_float)]
    L.ctsmg_batch_sync.argtypes = [C.c_void_p]
    L.ctsmg_batch_download.argtypes = [C.c_void_p, P(abi.SoilWaterIO), P(abi.SoilTempIO)]
    L.ctsmg_batch_autotune.argtypes = [C.c_void_p, C.c_int32, P(C.c_int32)]
    L.ctsmg_batch_set_block.argtypes = [C.c_void_p, C.c_int32]
    L.ctsmg_batch_state_bytes.argtypes = [C.c_void_p]
    L.ctsmg_batch_state_bytes.restype = C.c_int64
    L.ctsmg_batch_destroy.argtypes = [C.c_void_p]
    L._batch_bound = True


class SoilBatch:
    """Resident batch of columns advanced by SoilWater + SoilTemperature steps."""

    def __init__(self, state, npatch, dtime=1800.0, e_ice=6.0, snow_thermal_cond_method=0):
        self.L = load()
        _bind(self.L)
        self.state = state
        self.ncol = state["zwt"].shape[0]
        self.npatch = npatch
        self._sw = abi.make_io(abi.SoilWaterIO, abi.SOILWATER_FIELDS, state, self.ncol)
        self._st = abi.make_io(abi.SoilTempIO, abi.SOILTEMP_FIELDS, state, self.ncol, npatch)
        self.h = C.c_void_p()
        check(self.L.ctsmg_batch_create(C.byref(self.h), C.byref(self._sw), C.byref(self._st), self.ncol, npatch,
                                        dtime, e_ice, snow_thermal_cond_method))

    def run(self, nsteps, timed=False):
        if timed:
            ms = (C.c_float * nsteps)()
            check(self.L.ctsmg_batch_run(self.h, nsteps, ms))
            return np.array(ms[:], dtype=np.float64)
        check(self.L.ctsmg_batch_run(self.h, nsteps, None))
        return None

    def sync(self):
        check(self.L.ctsmg_batch_sync(self.h))

    def download(self, state=None):
        st = state if state is not None else self.state
        sw = abi.make_io(abi.SoilWaterIO, abi.SOILWATER_FIELDS, st, self.ncol)
        tt = abi.make_io(abi.SoilTempIO, abi.SOILTEMP_FIELDS, st, self.ncol, self.npatch)
        check(self.L.ctsmg_batch_download(self.h, C.byref(sw), C.byref(tt)))
        return st

    def autotune(self, trial_steps=2):
        b = C.c_int32()
        check(self.L.ctsmg_batch_autotune(self.h, trial_steps, C.byref(b)))
        return b.value

    def set_block(self, block):
        check(self.L.ctsmg_batch_set_block(self.h, block))

    def state_bytes(self):
        return int(self.L.ctsmg_batch_state_bytes(self.h))

    def close(self):
        if self.h:
            self.L.ctsmg_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
