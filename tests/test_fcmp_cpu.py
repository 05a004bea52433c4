"""The integer-pipe comparisons, min and max of ctsm_gb300/csrc/fcmp.cuh,
host build: every form agrees with the host's IEEE comparison (and fmin /
fmax, NaN operands yielding the other operand) on the edge cases and on 2^22
random pairs.  The device build is compared with the device's FP64
instructions in tests/test_fcmp_gpu.py."""
import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "ctsm_gb300", "csrc")


def test_host_fcmp_matches_ieee(tmp_path):
    so = os.path.join(str(tmp_path), "fcmp_host.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", CSRC,
                    os.path.join(HERE, "fcmp_host.cpp"), "-o", so], check=True)
    lib = C.CDLL(so)
    lib.fcmp_check.argtypes = [C.c_longlong, C.c_ulonglong]
    lib.fcmp_check.restype = C.c_longlong
    assert lib.fcmp_check(1 << 22, 987654321) == 0
