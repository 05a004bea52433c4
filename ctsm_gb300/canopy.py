"""Host-side mirror of the reference's CanopyFluxes interface (one dict of
numpy arrays stands for the derived types; every call goes through the C-ABI
of libctsm_gpu.so)."""
import ctypes as C

import numpy as np

from . import abi, canopy_inputs
from ._lib import load, check


def _bind(L):
    if getattr(L, "_canopy_bound", False):
        return
    L.ctsmg_set_canopy_params.argtypes = [C.POINTER(abi.CanopyParams), C.POINTER(abi.Pftcon)]
    L.ctsmg_canopyfluxes.argtypes = [C.POINTER(abi.Bounds), C.c_int32, C.POINTER(C.c_int32),
                                     C.POINTER(abi.CanopyIO), C.c_double]
    L._canopy_bound = True


def set_params(params=None, pftcon=None):
    """ctsmg_set_canopy_params: readParams of CanopyFluxesMod / PhotosynthesisMod
    and the pftcon arrays (defaults: ctsm_gb300.canopy_inputs)."""
    L = load()
    _bind(L)
    p = params if params is not None else canopy_inputs.make_params()
    f = pftcon if pftcon is not None else canopy_inputs.make_pftcon()
    check(L.ctsmg_set_canopy_params(C.byref(p), C.byref(f)))


def CanopyFluxes(bounds, num_exposedvegp, filter_exposedvegp, state, dtime, ngrid, begg=1):
    """CanopyFluxes (CanopyFluxesMod.F90:191) over the exposed-vegetation filter."""
    L = load()
    _bind(L)
    f = np.ascontiguousarray(filter_exposedvegp, dtype=np.int32)
    ncol = bounds.endc - bounds.begc + 1
    npat = bounds.endp - bounds.begp + 1
    io = abi.make_io(abi.CanopyIO, abi.CANOPY_FIELDS, state, ncol, npat, ngrid, begg)
    check(L.ctsmg_canopyfluxes(C.byref(bounds), int(num_exposedvegp), f.ctypes.data_as(C.POINTER(C.c_int32)),
                               C.byref(io), float(dtime)))


def RootMoistStress(bounds, num_exposedvegp, filter_exposedvegp, state):
    """The root moisture stress CanopyFluxes computes before its iteration
    (CanopyFluxesMod.F90:833-895 -> calc_root_moist_stress,
    SoilMoistStressMod.F90:438-514): eff_porosity, h2osoi_liqvol, btran,
    rootr and rresis of `state` are written."""
    L = load()
    if not getattr(L, "_rootmoist_bound", False):
        L.ctsmg_root_moist_stress.argtypes = [C.POINTER(abi.Bounds), C.c_int32, C.POINTER(C.c_int32),
                                              C.POINTER(abi.RootMoistIO)]
        L._rootmoist_bound = True
    f = np.ascontiguousarray(filter_exposedvegp, dtype=np.int32)
    ncol = bounds.endc - bounds.begc + 1
    npat = bounds.endp - bounds.begp + 1
    io = abi.make_io(abi.RootMoistIO, abi.ROOTMOIST_FIELDS, state, ncol, npat)
    check(L.ctsmg_root_moist_stress(C.byref(bounds), int(num_exposedvegp), f.ctypes.data_as(C.POINTER(C.c_int32)),
                                    C.byref(io)))


def BareGroundFluxes(bounds, num_noexposedvegp, filter_noexposedvegp, state, ngrid, begg=1):
    """BareGroundFluxes (BareGroundFluxesMod.F90:73) over the patches without
    exposed vegetation; the soil resistance method of soil.set_soil_resistance
    selects soilresis (sl_14) or soilbeta."""
    L = load()
    _bind(L)
    if not getattr(L, "_bare_bound", False):
        L.ctsmg_baregroundfluxes.argtypes = [C.POINTER(abi.Bounds), C.c_int32, C.POINTER(C.c_int32),
                                             C.POINTER(abi.BareGrndIO)]
        L._bare_bound = True
    f = np.ascontiguousarray(filter_noexposedvegp, dtype=np.int32)
    ncol = bounds.endc - bounds.begc + 1
    npat = bounds.endp - bounds.begp + 1
    io = abi.make_io(abi.BareGrndIO, abi.BAREGRND_FIELDS, state, ncol, npat, ngrid, begg)
    check(L.ctsmg_baregroundfluxes(C.byref(bounds), int(num_noexposedvegp), f.ctypes.data_as(C.POINTER(C.c_int32)),
                                   C.byref(io)))

