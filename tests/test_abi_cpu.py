"""The C-ABI library builds, loads without a GPU, exports every function
include/ctsm_gpu.h declares, and its struct layouts match the ctypes mirror."""
import ctypes as C
import os
import re
import subprocess

import pytest

from ctsm_gb300 import abi
from ctsm_gb300.engine import BatchConfig, BatchInputs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ctsm_gpu.h")


def declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\**(ctsmg_\w+)\s*\(", txt, re.M)))


@pytest.fixture(scope="module")
def lib():
    from ctsm_gb300 import build
    path = build.build()
    return C.CDLL(path)


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 12
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_init_without_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib.ctsmg_init.argtypes = [C.POINTER(abi.Options)]
    lib.ctsmg_last_error.restype = C.c_char_p
    rc = lib.ctsmg_init(C.byref(abi.Options(0, 0, 40, 1, 12, 20, 25)))
    assert rc == 2          # CTSMG_E_CUDA: no device
    assert lib.ctsmg_last_error()


def test_unsupported_options_rejected(lib):
    lib.ctsmg_init.argtypes = [C.POINTER(abi.Options)]
    assert lib.ctsmg_init(C.byref(abi.Options(2, 0, 40, 1, 12, 20, 25))) == 10   # mixed form is empty
    assert lib.ctsmg_init(C.byref(abi.Options(0, 0, 40, 1, 10, 20, 25))) == 10   # nlevsno must be 12


def test_struct_layout_matches_ctypes(tmp_path):
    """Compile a C probe against the header and compare sizeof/offsetof."""
    fields = {"ctsmg_soilwater_io": (abi.SoilWaterIO, ["ldc"] + [f[0] for f in abi.SOILWATER_FIELDS +
                                                                    abi.SOILWATER_EXTRA]),
              "ctsmg_soilwater_movement_nml": (abi.SoilWaterMovementNml,
                                               [f[0] for f in abi.SoilWaterMovementNml._fields_]),
              "ctsmg_baregrnd_io": (abi.BareGrndIO, ["ldp", "ldc", "ldg", "begg"] +
                                    [f[0] for f in abi.BAREGRND_FIELDS]),
              "ctsmg_hydrology_io": (abi.HydrologyIO, ["ldc"] + [f[0] for f in abi.HYDROLOGY_FIELDS]),
              "ctsmg_soilhydrology_params": (abi.SoilHydrologyParams,
                                             [f[0] for f in abi.SoilHydrologyParams._fields_]),
              "ctsmg_soilresis_io": (abi.SoilResisIO, ["ldc"] + [f[0] for f in abi.SOILRESIS_FIELDS]),
              "ctsmg_soil_resistance_params": (abi.SoilResistanceParams,
                                               [f[0] for f in abi.SoilResistanceParams._fields_]),
              "ctsmg_soiltemp_io": (abi.SoilTempIO, ["ldc", "ldp"] + [f[0] for f in abi.SOILTEMP_FIELDS]),
              "ctsmg_soilfluxes_io": (abi.SoilFluxesIO, ["ldc", "ldp"] + [f[0] for f in abi.SOILFLUXES_FIELDS]),
              "ctsmg_rootmoist_io": (abi.RootMoistIO, ["ldc", "ldp"] + [f[0] for f in abi.ROOTMOIST_FIELDS]),
              "ctsmg_pftcon": (abi.Pftcon, [f[0] for f in abi.Pftcon._fields_]),
              "ctsmg_canopy_io": (abi.CanopyIO, ["ldp", "ldc", "ldg", "begg"] + [f[0] for f in abi.CANOPY_FIELDS]),
              "ctsmg_batch_config": (BatchConfig, [f[0] for f in BatchConfig._fields_]),
              "ctsmg_batch_inputs": (BatchInputs, [f[0] for f in BatchInputs._fields_]),
              "ctsmg_bounds": (abi.Bounds, ["begc", "endc", "begp", "endp"]),
              "ctsmg_options": (abi.Options, [f[0] for f in abi.Options._fields_])}
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "ctsm_gpu.h"', "int main(void){"]
    for s, (_, names) in fields.items():
        src.append('printf("%s %%zu\\n", sizeof(%s));' % (s, s))
        for n in names:
            src.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (s, n, s, n))
    src.append("return 0;}")
    c = tmp_path / "probe.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe)], check=True)
    out = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], capture_output=True,
                                                               text=True).stdout.splitlines())
    for s, (cls, names) in fields.items():
        assert int(out[s]) == C.sizeof(cls), s
        for n in names:
            assert int(out[s + "." + n]) == getattr(cls, n).offset, (s, n)
