"""Builds tests/fastmath_host.cpp with g++ (no contraction) and evaluates the
kernels' log / log10 / exp / pow on the host: out rows log(x), log10(x),
exp(y), pow(x, y)."""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "ctsm_gb300", "csrc")


def build(outdir):
    so = os.path.join(str(outdir), "fastmath_host.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I", CSRC,
                    os.path.join(HERE, "fastmath_host.cpp"), "-o", so], check=True)
    lib = C.CDLL(so)
    P = C.POINTER(C.c_double)
    lib.fm_eval.argtypes = [C.c_int, P, P, P]
    return lib


def evaluate(lib, x, y):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    out = np.empty(4 * len(x))
    P = C.POINTER(C.c_double)
    lib.fm_eval(len(x), x.ctypes.data_as(P), y.ctypes.data_as(P), out.ctypes.data_as(P))
    return out.reshape(4, len(x))
