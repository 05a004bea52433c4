"""ctypes loader for oracle/liboracle.so (built by oracle/Makefile)."""
import ctypes as C
import os
import subprocess

from ctsm_gb300 import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def build(force=False):
    so = os.path.join(_HERE, "liboracle.so")
    if force or not os.path.exists(so) or any(
            os.path.getmtime(os.path.join(_HERE, f)) > os.path.getmtime(so)
            for f in os.listdir(_HERE) if f.endswith((".cpp", ".h"))):
        subprocess.run(["make", "-s", "-C", _HERE, "-B" if force else "all"], check=True)
    return so


def lib():
    global _LIB
    if _LIB is None:
        _LIB = C.CDLL(build())
        P, I = C.POINTER, C.c_int
        _LIB.oracle_soilwater.argtypes = [P(abi.Bounds), I, P(C.c_int32), P(abi.SoilWaterIO), C.c_double, C.c_double]
        _LIB.oracle_soiltemperature.argtypes = [P(abi.Bounds), I, P(C.c_int32), P(abi.SoilTempIO), C.c_double, I]
        _LIB.oracle_dgbsv.argtypes = [I, I, I, P(C.c_double), I, P(C.c_int), P(C.c_double)]
        _LIB.oracle_tridiagonal.argtypes = [I] + [P(C.c_double)] * 5
        _LIB.oracle_tridiagonal.restype = None
        _LIB.oracle_set_libm_noise.argtypes = [I, C.c_ulonglong]
        _LIB.oracle_set_libm_noise.restype = None
        _LIB.oracle_set_canopy_params.argtypes = [P(abi.CanopyParams), P(abi.Pftcon), I, I]
        _LIB.oracle_set_canopy_params.restype = None
        _LIB.oracle_quadratic.argtypes = [C.c_double] * 3 + [P(C.c_double)] * 2
        _LIB.oracle_qsat.argtypes = [C.c_double, C.c_double] + [P(C.c_double)] * 3
        _LIB.oracle_qsat.restype = None
        _LIB.oracle_set_patch_medlyn.argtypes = [P(C.c_double), P(C.c_double)]
        _LIB.oracle_set_patch_medlyn.restype = None
        _LIB.oracle_rootsink.argtypes = [I, I, P(C.c_int32), P(C.c_int32)] + [P(C.c_double)] * 4
        _LIB.oracle_rootsink.restype = None
        _LIB.oracle_root_sink.argtypes = [P(abi.Bounds), I, P(C.c_int32), P(abi.RootSinkIO)]
        _LIB.oracle_canopyfluxes.argtypes = [P(abi.Bounds), I, P(C.c_int32), P(abi.CanopyIO), C.c_double, P(C.c_int)]
        _LIB.oracle_hydrology.argtypes = [P(abi.Bounds), I, P(C.c_int32), P(abi.HydrologyIO), I,
                                          P(abi.SoilHydrologyParams), C.c_double]
        _LIB.oracle_baregroundfluxes.argtypes = [P(abi.Bounds), I, P(C.c_int32), P(abi.BareGrndIO), I]
        _LIB.oracle_soilevap_resis.argtypes = [P(abi.Bounds), I, P(C.c_int32), P(abi.SoilResisIO),
                                               P(abi.SoilResistanceParams)]
        _LIB.oracle_dgtsv.argtypes = [I] + [P(C.c_double)] * 4
        _LIB.oracle_soilwater_mf.argtypes = [P(abi.Bounds), I, P(C.c_int32), P(abi.SoilWaterIO), C.c_double,
                                             C.c_double, P(abi.SoilWaterMovementNml), P(C.c_int)]
        _LIB.oracle_flexcn_fix.argtypes = [P(abi.Bounds), I, P(C.c_int32), P(abi.SoilWaterIO)]
        _LIB.oracle_flexcn_fix.restype = None
        _LIB.oracle_set_soil_water_fractions.argtypes = [P(abi.Bounds), I, P(C.c_int32), P(abi.SoilWaterIO)]
        _LIB.oracle_set_soil_water_fractions.restype = None
        _LIB.oracle_root_moist_stress.argtypes = [P(abi.Bounds), I, P(C.c_int32), P(abi.RootMoistIO)]
        _LIB.oracle_soilfluxes.argtypes = [P(abi.Bounds), I, P(C.c_int32), I, P(C.c_int32), P(abi.SoilFluxesIO),
                                           C.c_double]
    return _LIB


def set_threads(n):
    os.environ["OMP_NUM_THREADS"] = str(n)
