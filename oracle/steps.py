"""Multi-step drivers of the oracle (test infrastructure): the sequences the
batched engine runs, stepped on the CPU."""
import ctypes as C

import numpy as np

from ctsm_gb300 import abi, inputs, canopy_inputs
from oracle import oracle as orc

DT = 1800.0


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def full_steps(A, npatch, ngrid, rootr, nsteps, medlyn_per_patch=False, method=1, itmax=40, snow_method=0,
               soilfluxes=False, rootmoist=False, swm=None, soilresis=None, hydro=None):
    """nsteps x (CanopyFluxes, root sink, SoilTemperature, [SoilFluxes,]
    SoilWater, h2osoi_vol refresh) in place on A.  displa / z0mv keep their
    SatellitePhenology values and cgrnds / cgrndl restart from zero every
    step; with soilfluxes the temperatures before SoilTemperature go to
    tssbef / t_h2osfc_bef; with rootmoist btran and rootr come from the root
    moisture stress of the current soil state at the start of every step
    (A then holds the ROOTMOIST components; `rootr` is not used).  swm (an
    abi.SoilWaterMovementNml) selects the SoilWater form and the flexibleCN
    fix; None is the Zeng-Decker form.  soilresis = [(column filter,
    abi.SoilResistanceParams), ...] runs calc_soilevap_resis first in every
    step (one entry per parameter set, e.g. per ensemble member); hydro (see
    `hydrology`) runs the default hydrology around SoilWater."""
    L = orc.lib()
    ncol = A["zwt"].shape[0]
    L.oracle_set_canopy_params(C.byref(canopy_inputs.make_params()), C.byref(canopy_inputs.make_pftcon()), method,
                               itmax)
    if medlyn_per_patch:
        L.oracle_set_patch_medlyn(_p(A["medlynslope_p"]), _p(A["medlynintercept_p"]))
    b = abi.Bounds(1, ncol, 1, npatch)
    filt_c = np.arange(1, ncol + 1, dtype=np.int32)
    filt_p = np.arange(1, npatch + 1, dtype=np.int32)
    displa0, z0mv0 = A["displa"].copy(), A["z0mv"].copy()
    rootr = np.ascontiguousarray(rootr)
    try:
        for _ in range(nsteps):
            A["displa"][:] = displa0
            A["z0mv"][:] = z0mv0
            A["cgrnds"][:] = 0.0
            A["cgrndl"][:] = 0.0
            if soilresis:
                sr = abi.make_io(abi.SoilResisIO, abi.SOILRESIS_FIELDS, A, ncol)
                for f, par in soilresis:
                    f = np.ascontiguousarray(f, dtype=np.int32)
                    assert L.oracle_soilevap_resis(C.byref(b), len(f), _p(f, C.c_int32), C.byref(sr), C.byref(par)) == 0
            if rootmoist:
                rm = abi.make_io(abi.RootMoistIO, abi.ROOTMOIST_FIELDS, A, ncol, npatch)
                assert L.oracle_root_moist_stress(C.byref(b), npatch, _p(filt_p, C.c_int32), C.byref(rm)) == 0
            ci = abi.make_io(abi.CanopyIO, abi.CANOPY_FIELDS, A, ncol, npatch, ngrid, 1)
            e = C.c_int(0)
            rc = L.oracle_canopyfluxes(C.byref(b), npatch, _p(filt_p, C.c_int32), C.byref(ci), DT, C.byref(e))
            assert rc == 0, (rc, e.value)
            L.oracle_rootsink(ncol, npatch, _p(A["col_patchi"], C.c_int32), _p(A["col_npatches"], C.c_int32),
                              _p(A["wtcol"]), _p(A["qflx_tran_veg"]), _p(A["rootr"] if rootmoist else rootr),
                              _p(A["qflx_rootsoi"]))
            if soilfluxes:
                A["tssbef"][:] = A["t_soisno"]
                A["t_h2osfc_bef"][:] = A["t_h2osfc"]
            st = abi.make_io(abi.SoilTempIO, abi.SOILTEMP_FIELDS, A, ncol, npatch)
            assert L.oracle_soiltemperature(C.byref(b), ncol, _p(filt_c, C.c_int32), C.byref(st), DT, snow_method) == 0
            if soilfluxes:
                sf = abi.make_io(abi.SoilFluxesIO, abi.SOILFLUXES_FIELDS, A, ncol, npatch)
                assert L.oracle_soilfluxes(C.byref(b), ncol, _p(filt_c, C.c_int32), npatch, _p(filt_p, C.c_int32),
                                           C.byref(sf), DT) == 0
            soilwater(L, A, b, filt_c, swm, hydro=hydro)
            inputs.refresh_h2osoi_vol(A)
    finally:
        A["displa"][:] = displa0
        A["z0mv"][:] = z0mv0
        if medlyn_per_patch:
            L.oracle_set_patch_medlyn(None, None)


def hydrology(L, A, b, filt_c, routines, hydro):
    """The default-hydrology routines `routines` (indices of oracle_hydrology)
    with hydro = [(column filter, abi.SoilHydrologyParams), ...] (one entry per
    parameter set, e.g. per ensemble member)."""
    ncol = A["zwt"].shape[0]
    io = abi.make_io(abi.HydrologyIO, abi.HYDROLOGY_FIELDS, A, ncol)
    for which in routines:
        for f, par in hydro:
            f = np.ascontiguousarray(f, dtype=np.int32)
            assert L.oracle_hydrology(C.byref(b), len(f), _p(f, C.c_int32), C.byref(io), which, C.byref(par), DT) == 0


def soilwater(L, A, b, filt_c, swm=None, e_ice=6.0, hydro=None):
    """HydrologyNoDrainage's SetSoilWaterFractions and SoilWater
    (HydrologyNoDrainageMod.F90:302, 346) in the form swm selects; with hydro
    (see `hydrology`) SaturatedExcessRunoff and the infiltration chain before
    SoilWater and the water tables and lateral flows after it (:308-368, HydrologyDrainageMod.F90:139-143)."""
    ncol = A["zwt"].shape[0]
    n = len(filt_c)
    fp = _p(filt_c, C.c_int32)
    aquifer = swm is None or swm.soilwater_movement_method == 0
    if aquifer:
        fields = abi.SOILWATER_FIELDS + ([x for x in abi.SOILWATER_EXTRA if x[0] in A] if swm is not None or hydro
                                         else [])
        sw = abi.make_io(abi.SoilWaterIO, fields, A, ncol)
        if hydro:
            L.oracle_set_soil_water_fractions(C.byref(b), n, fp, C.byref(sw))
            hydrology(L, A, b, filt_c, [0, 5], hydro)
        assert L.oracle_soilwater(C.byref(b), n, fp, C.byref(sw), e_ice, DT) == 0
    else:
        sw = abi.make_io(abi.SoilWaterIO, abi.SOILWATER_FIELDS + abi.SOILWATER_EXTRA, A, ncol)
        L.oracle_set_soil_water_fractions(C.byref(b), n, fp, C.byref(sw))
        if hydro:
            hydrology(L, A, b, filt_c, [0, 5], hydro)
        e = C.c_int(0)
        assert L.oracle_soilwater_mf(C.byref(b), n, fp, C.byref(sw), e_ice, DT, C.byref(swm), C.byref(e)) == 0, e.value
    if swm is not None and swm.use_flexibleCN:
        L.oracle_flexcn_fix(C.byref(b), n, fp, C.byref(sw))
    if hydro:       # WaterTable + Drainage after the Zeng-Decker form, the default hydrology after the moisture form
        hydrology(L, A, b, filt_c, [6, 7] if aquifer else [1, 2, 3, 4], hydro)


def soil_steps(A, npatch, nsteps, swm=None, snow_method=0, hydro=None):
    """nsteps x (SoilWater [with the default hydrology around it], SoilTemperature,
    h2osoi_vol refresh): the batched engine's order 0."""
    L = orc.lib()
    ncol = A["zwt"].shape[0]
    b = abi.Bounds(1, ncol, 1, npatch)
    filt = np.arange(1, ncol + 1, dtype=np.int32)
    st = abi.make_io(abi.SoilTempIO, abi.SOILTEMP_FIELDS, A, ncol, npatch)
    for _ in range(nsteps):
        soilwater(L, A, b, filt, swm, hydro=hydro)
        assert L.oracle_soiltemperature(C.byref(b), ncol, _p(filt, C.c_int32), C.byref(st), DT, snow_method) == 0
        inputs.refresh_h2osoi_vol(A)

