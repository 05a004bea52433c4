"""Host-side mirror of the reference's SoilWater / SoilTemperature interface.

The functions keep the reference's names and argument meaning (bounds,
filter length, 1-based filter, the derived-type components, dtime) and its
error behaviour (endrun becomes CtsmError carrying the same context).  The
derived types are represented by one dict of numpy arrays keyed by component
name, laid out as the Fortran arrays are: (levels, columns) C-contiguous, i.e.
columns fastest.  Every call goes through the C-ABI of libctsm_gpu.so."""
import ctypes as C

import numpy as np

from . import abi
from ._lib import load, check

_INIT = {}


def init(snow_thermal_cond_method=0, stomatalcond_method=1, itmax_canopy_fluxes=40, e_ice=6.0,
         soilwater_movement_method=0):
    """ctsmg_init + ctsmg_set_soilwater_params (the namelist and readParams
    steps of SoilWaterMovementMod.F90:89-216 and CanopyFluxesMod.F90:92-188)."""
    L = load()
    opt = abi.Options(soilwater_movement_method, snow_thermal_cond_method, itmax_canopy_fluxes, stomatalcond_method,
                      abi.NLEVSNO, abi.NLEVSOI, abi.NLEVGRND)
    check(L.ctsmg_init(C.byref(opt)))
    check(L.ctsmg_set_soilwater_params(C.byref(abi.SoilWaterParams(e_ice))))
    _INIT.update(snow_thermal_cond_method=snow_thermal_cond_method, e_ice=e_ice)


def set_soilwater_movement(nml):
    """ctsmg_set_soilwater_movement: the soilwater_movement_inparm namelist
    (init_soilwater_movement, SoilWaterMovementMod.F90:108-216); build it with
    abi.soilwater_movement_nml."""
    check(load().ctsmg_set_soilwater_movement(C.byref(nml)))


def _filter(filt):
    f = np.ascontiguousarray(filt, dtype=np.int32)
    return f, f.ctypes.data_as(C.POINTER(C.c_int32))


def SoilWater(bounds, num_hydrologyc, filter_hydrologyc, state, dtime):
    """SoilWater (SoilWaterMovementMod.F90:240) in the form the namelist
    selects; the moisture form and the flexibleCN fix also take the
    SOILWATER_EXTRA components of `state`."""
    L = load()
    f, fp = _filter(filter_hydrologyc)
    ncol = bounds.endc - bounds.begc + 1
    fields = abi.SOILWATER_FIELDS + [x for x in abi.SOILWATER_EXTRA if x[0] in state]
    io = abi.make_io(abi.SoilWaterIO, fields, state, ncol)
    check(L.ctsmg_soilwater(C.byref(bounds), int(num_hydrologyc), fp, C.byref(io), float(dtime)))


def SoilTemperature(bounds, num_nolakec, filter_nolakec, state, dtime):
    """SoilTemperature (SoilTemperatureMod.F90:92) for natural-vegetation columns."""
    L = load()
    f, fp = _filter(filter_nolakec)
    ncol = bounds.endc - bounds.begc + 1
    npat = bounds.endp - bounds.begp + 1
    io = abi.make_io(abi.SoilTempIO, abi.SOILTEMP_FIELDS, state, ncol, npat)
    check(L.ctsmg_soiltemperature(C.byref(bounds), int(num_nolakec), fp, C.byref(io), float(dtime)))


def RootSink(bounds, num_filterc, filterc, state, tran_col=True):
    """Compute_EffecRootFrac_And_VertTranSink_Default
    (SoilWaterPlantSinkMod.F90:332) over the column filter; tran_col=False
    passes no qflx_tran_veg_col (the library then uses the wtcol-weighted sum
    of the patches' transpiration)."""
    L = load()
    L.ctsmg_root_sink.argtypes = [C.POINTER(abi.Bounds), C.c_int32, C.POINTER(C.c_int32),
                                  C.POINTER(abi.RootSinkIO)]
    f, fp = _filter(filterc)
    ncol = bounds.endc - bounds.begc + 1
    npat = bounds.endp - bounds.begp + 1
    fields = [x for x in abi.ROOTSINK_FIELDS if tran_col or x[0] != "qflx_tran_veg_col"]
    io = abi.make_io(abi.RootSinkIO, fields, state, ncol, npat)
    check(L.ctsmg_root_sink(C.byref(bounds), int(num_filterc), fp, C.byref(io)))


def SoilFluxes(bounds, num_nolakec, filter_nolakec, num_nolakep, filter_nolakep, state, dtime):
    """SoilFluxes (SoilFluxesMod.F90:36) after SoilTemperature; `state` also
    holds tssbef / t_h2osfc_bef, the temperatures saved before SoilTemperature."""
    L = load()
    fc, fcp = _filter(filter_nolakec)
    fp, fpp = _filter(filter_nolakep)
    ncol = bounds.endc - bounds.begc + 1
    npat = bounds.endp - bounds.begp + 1
    io = abi.make_io(abi.SoilFluxesIO, abi.SOILFLUXES_FIELDS, state, ncol, npat)
    check(L.ctsmg_soilfluxes(C.byref(bounds), int(num_nolakec), fcp, int(num_nolakep), fpp, C.byref(io), float(dtime)))


def set_soil_resistance(method=1, d_max=15.0, frac_sat_soil_dsl_init=0.8):
    """ctsmg_set_soil_resistance: soil_resis_method (1 sl_14, 0 leepielke_1992)
    and the parameter-file values d_max (mm) and frac_sat_soil_dsl_init
    (SurfaceResistanceMod.F90:60-111)."""
    L = load()
    L.ctsmg_set_soil_resistance.argtypes = [C.POINTER(abi.SoilResistanceParams)]
    check(L.ctsmg_set_soil_resistance(C.byref(abi.SoilResistanceParams(method, d_max, frac_sat_soil_dsl_init))))


def calc_soilevap_resis(bounds, num_nolakec, filter_nolakec, state):
    """calc_soilevap_resis (SurfaceResistanceMod.F90:190) over the column filter."""
    L = load()
    L.ctsmg_soilevap_resis.argtypes = [C.POINTER(abi.Bounds), C.c_int32, C.POINTER(C.c_int32),
                                       C.POINTER(abi.SoilResisIO)]
    f, fp = _filter(filter_nolakec)
    ncol = bounds.endc - bounds.begc + 1
    io = abi.make_io(abi.SoilResisIO, abi.SOILRESIS_FIELDS, state, ncol)
    check(L.ctsmg_soilevap_resis(C.byref(bounds), int(num_nolakec), fp, C.byref(io)))


HYDROLOGY_ROUTINES = ("WaterTable", "Drainage", "SaturatedExcessRunoff", "InfiltrationChain", "PerchedWaterTable", "ThetaBasedWaterTable", "PerchedLateralFlow",
                      "SubsurfaceLateralFlow")
_HYD_ENTRY = {"SaturatedExcessRunoff": "ctsmg_saturated_excess_runoff",
              "InfiltrationChain": "ctsmg_infiltration_chain",
              "WaterTable": "ctsmg_water_table",
              "Drainage": "ctsmg_drainage",
              "PerchedWaterTable": "ctsmg_perched_water_table",
              "ThetaBasedWaterTable": "ctsmg_theta_based_water_table",
              "PerchedLateralFlow": "ctsmg_perched_lateral_flow",
              "SubsurfaceLateralFlow": "ctsmg_subsurface_lateral_flow"}


def set_soilhydrology_params(aq_sp_yield_min=0.01, n_baseflow=1.0, baseflow_scalar=1.0e-2,
                             perched_baseflow_scalar=1.0e-5, e_ice=6.0, fff=0.5, pc=0.4, mu=0.13, h2osfcflag=1):
    """ctsmg_set_soilhydrology_params: readParams of SoilHydrologyMod
    (SoilHydrologyMod.F90:174-199), SaturatedExcessRunoffMod (fff) and
    SurfaceWaterMod (pc, mu), and h2osfcflag.  The parameter-file values are
    builder's choices (the file is absent)."""
    L = load()
    L.ctsmg_set_soilhydrology_params.argtypes = [C.POINTER(abi.SoilHydrologyParams)]
    p = abi.SoilHydrologyParams(aq_sp_yield_min, n_baseflow, baseflow_scalar, perched_baseflow_scalar, e_ice, fff,
                                pc, mu, h2osfcflag)
    check(L.ctsmg_set_soilhydrology_params(C.byref(p)))


def hydrology(routine, bounds, num_hydrologyc, filter_hydrologyc, state, dtime=None):
    """One of the water-table / drainage routines (HYDROLOGY_ROUTINES, by the
    reference's subroutine name) over the column filter."""
    L = load()
    name = _HYD_ENTRY[routine]
    fn = getattr(L, name)
    args = [C.POINTER(abi.Bounds), C.c_int32, C.POINTER(C.c_int32), C.POINTER(abi.HydrologyIO)]
    lateral = routine not in ("SaturatedExcessRunoff", "PerchedWaterTable", "ThetaBasedWaterTable")
    fn.argtypes = args + ([C.c_double] if lateral else [])
    f, fp = _filter(filter_hydrologyc)
    ncol = bounds.endc - bounds.begc + 1
    io = abi.make_io(abi.HydrologyIO, abi.HYDROLOGY_FIELDS, state, ncol)
    extra = [float(dtime)] if lateral else []
    check(fn(C.byref(bounds), int(num_hydrologyc), fp, C.byref(io), *extra))

