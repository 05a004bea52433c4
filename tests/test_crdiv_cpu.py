"""The shared-reciprocal quotient of ctsm_gb300/csrc/cr_div.cuh (one
Newton-Markstein correction of a * RN(1/b)) gives the bits of the IEEE
division except where a/b lies within 2^-103.9 |a/b| of a rounding midpoint
-- a set that random pairs essentially never hit: 4 x 2^22 pairs on the host
build (random bits over the whole double range, physical magnitudes, divisors
with all-ones significands, quotients within a few ulp of rounding midpoints)
match the division bit for bit.  The device build is compared with the device
division in tests/test_crdiv_gpu.py."""
import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "ctsm_gb300", "csrc")


def test_host_crdiv_equals_division(tmp_path):
    so = os.path.join(str(tmp_path), "crdiv_host.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I", CSRC,
                    os.path.join(HERE, "crdiv_host.cpp"), "-o", so], check=True)
    lib = C.CDLL(so)
    lib.crdiv_check.argtypes = [C.c_longlong, C.c_ulonglong, C.c_int]
    lib.crdiv_check.restype = C.c_longlong
    for mode in range(4):
        assert lib.crdiv_check(1 << 22, 1234567 + mode, mode) == 0, mode
