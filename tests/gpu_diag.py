"""Builds and loads tests/gpu_diag.cu, the test-only library of device-math
diagnostics (nvcc, sm_103a), into tests/_build/."""
import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "ctsm_gb300", "csrc")
OUT = os.path.join(HERE, "_build")
SO = os.path.join(OUT, "libctsm_diag.so")
_LIB = None


def build(force=False):
    from ctsm_gb300 import build as b
    src = os.path.join(HERE, "gpu_diag.cu")
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    if not force and os.path.exists(SO) and all(os.path.getmtime(d) <= os.path.getmtime(SO) for d in deps):
        return SO
    os.makedirs(OUT, exist_ok=True)
    cmd = [b.nvcc()] + b.ARCH + ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
                                 "-I" + os.path.join(ROOT, "include"), "-I" + CSRC, src, "-o", SO + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(SO + ".tmp", SO)
    return SO


def load():
    global _LIB
    if _LIB is None:
        _LIB = C.CDLL(build())
        P = C.POINTER(C.c_double)
        _LIB.ctsmg_diag_fastmath.argtypes = [C.c_int32, P, P, P]
        _LIB.ctsmg_diag_powers.argtypes = [C.c_int32, P, P, P]
        _LIB.ctsmg_diag_crdiv.argtypes = [C.c_int32, P, P, P]
        _LIB.ctsmg_diag_fcmp.argtypes = [C.c_int32, P, P, P]
    return _LIB


def check(rc):
    if rc != 0:
        raise RuntimeError("diagnostic call failed with status %d" % rc)
