"""ctypes binding of libctsm_gpu.so.  There is no CPU fallback: if the library
is missing or was not built, loading raises."""
import ctypes as C
import os

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libctsm_gpu.so")
_LIB = None


class CtsmError(RuntimeError):
    """Raised where the reference calls endrun; carries the status code and
    the (column or patch, level) context."""

    def __init__(self, code, msg, index=0, level=0):
        super().__init__("ctsm_gpu error %d: %s (index %d, level %d)" % (code, msg, index, level))
        self.code, self.index, self.level = code, index, level


def load():
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libctsm_gpu.so is not built (run __graft_entry__.build()); "
                           "the CUDA library is required, there is no CPU path")
    L = C.CDLL(LIB_PATH)
    P = C.POINTER
    L.ctsmg_init.argtypes = [P(abi.Options)]
    L.ctsmg_set_soilwater_params.argtypes = [P(abi.SoilWaterParams)]
    L.ctsmg_set_soilwater_movement.argtypes = [P(abi.SoilWaterMovementNml)]
    L.ctsmg_last_error.restype = C.c_char_p
    L.ctsmg_last_error_index.argtypes = [P(C.c_int32), P(C.c_int32)]
    L.ctsmg_soilwater.argtypes = [P(abi.Bounds), C.c_int32, P(C.c_int32), P(abi.SoilWaterIO), C.c_double]
    L.ctsmg_soiltemperature.argtypes = [P(abi.Bounds), C.c_int32, P(C.c_int32), P(abi.SoilTempIO), C.c_double]
    L.ctsmg_soilfluxes.argtypes = [P(abi.Bounds), C.c_int32, P(C.c_int32), C.c_int32, P(C.c_int32),
                                   P(abi.SoilFluxesIO), C.c_double]
    _LIB = L
    return L


def check(rc):
    if rc != 0:
        L = load()
        i, l = C.c_int32(), C.c_int32()
        L.ctsmg_last_error_index(C.byref(i), C.byref(l))
        raise CtsmError(rc, L.ctsmg_last_error().decode(), i.value, l.value)
    return rc
