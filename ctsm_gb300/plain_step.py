"""The plain form of a model step: what a CTSM host does with the drop-in
calls alone -- CanopyFluxes, the root water sink, SoilTemperature, SoilWater
and the between-step h2osoi_vol refresh, each call copying its arrays from
and back to host memory (src/main/clm_driver.F90:766, 900, 950; the sink of
src/biogeophys/SoilWaterPlantSinkMod.F90:332-420 and the refresh of
src/biogeophys/HydrologyNoDrainageMod.F90:580,590 run on the host, as they
do in the reference).  It is the baseline the batched engine is compared
with: one member or region per set of calls, no state kept on the device."""
import numpy as np

from . import abi, canopy, canopy_inputs, inputs, soil

DT = 1800.0


def root_sink(A, rootr):
    """qflx_rootsoi (levels 1..nlevsoi, columns) from the patches' transpiration
    and root fractions, summed over each column's patches in patch order."""
    ncol = A["zwt"].shape[0]
    npch = A["wtcol"].shape[0]
    pcol = np.repeat(np.arange(ncol), A["col_npatches"])
    tw = A["qflx_tran_veg"] * A["wtcol"]
    rc = np.zeros((abi.NLEVSOI, ncol))
    for j in range(abi.NLEVSOI):
        rc[j] = np.bincount(pcol, weights=rootr[j, :npch] * A["qflx_tran_veg"] * A["wtcol"], minlength=ncol)
    temp = np.bincount(pcol, weights=tw, minlength=ncol)
    rc = np.where(temp != 0.0, rc / np.where(temp != 0.0, temp, 1.0), rc)
    A["qflx_rootsoi"][...] = rc * temp


def full_step(A, npatch, ngrid, rootr, displa0, z0mv0, medlyn=None, params=None):
    """One plain full step in place on A.  medlyn = (slope, intercept) factors
    of an ensemble member, applied through the pftcon rows (the drop-in reads
    the parameters from pftcon)."""
    ncol = A["zwt"].shape[0]
    if medlyn is not None:
        rows = [list(r) for r in canopy_inputs.DEFAULT_PFT]
        for r in rows:
            r[6] *= medlyn[0]
            r[7] *= medlyn[1]
        canopy.set_params(params, canopy_inputs.make_pftcon(rows))
    A["displa"][:] = displa0
    A["z0mv"][:] = z0mv0
    A["cgrnds"][:] = 0.0
    A["cgrndl"][:] = 0.0
    b = abi.Bounds(1, ncol, 1, npatch)
    canopy.CanopyFluxes(b, npatch, np.arange(1, npatch + 1, dtype=np.int32), A, DT, ngrid)
    root_sink(A, rootr)
    filt = np.arange(1, ncol + 1, dtype=np.int32)
    soil.SoilTemperature(b, ncol, filt, A, DT)
    soil.SoilWater(b, ncol, filt, A, DT)
    inputs.refresh_h2osoi_vol(A)


class PlainCLM5Step:
    """The CLM5-default step of one ensemble member (or region) made of
    drop-in calls through the C-ABI alone, in the driver's order
    (src/main/clm_driver.F90:700-960, HydrologyNoDrainageMod.F90:302-372,
    HydrologyDrainageMod.F90:139-143): soil evaporative resistance, root
    moisture stress, CanopyFluxes, the root sink, SoilTemperature, SoilFluxes,
    SetSoilWaterFractions, SaturatedExcessRunoff, the infiltration chain,
    SoilWater (moisture form), the perched and theta-based water tables, the
    perched and subsurface lateral flows.  Each call copies its arrays from and
    back to host memory; the member's parameters go in through the setters
    (pftcon Medlyn rows, d_max, baseflow_scalar and fff) before its calls.
    Between calls the host only saves the temperatures SoilFluxes needs,
    restores the SatellitePhenology roughness and refreshes h2osoi_vol, as the
    reference's driver does.  The io structs are built once."""

    def __init__(self, S, npatch, ngrid, medlyn=(1.0, 1.0), d_max=15.0, baseflow_scalar=1.0e-2, fff=0.5,
                 params=None):
        import ctypes as C
        from ._lib import load
        self.C = C
        self.L = L = load()
        canopy._bind(L)
        self.S = S
        ncol = S["zwt"].shape[0]
        self.ncol, self.npatch, self.ngrid = ncol, npatch, ngrid
        self.b = abi.Bounds(1, ncol, 1, npatch)
        self.fc = np.arange(1, ncol + 1, dtype=np.int32)
        self.fp = np.arange(1, npatch + 1, dtype=np.int32)
        P32 = C.POINTER(C.c_int32)
        self.pfc, self.pfp = self.fc.ctypes.data_as(P32), self.fp.ctypes.data_as(P32)
        rows = [list(r) for r in canopy_inputs.DEFAULT_PFT]
        for r in rows:
            r[6] *= medlyn[0]
            r[7] *= medlyn[1]
        self.par = params if params is not None else canopy_inputs.make_params()
        self.pft = canopy_inputs.make_pftcon(rows)
        self.sres = abi.SoilResistanceParams(1, d_max, 0.8)
        self.hyd = abi.SoilHydrologyParams(0.01, 1.0, baseflow_scalar, 1.0e-5, 6.0, fff, 0.4, 0.13, 1)
        self.io = {
            "sr": abi.make_io(abi.SoilResisIO, abi.SOILRESIS_FIELDS, S, ncol),
            "rm": abi.make_io(abi.RootMoistIO, abi.ROOTMOIST_FIELDS, S, ncol, npatch),
            "ci": abi.make_io(abi.CanopyIO, abi.CANOPY_FIELDS, S, ncol, npatch, ngrid, 1),
            "rs": abi.make_io(abi.RootSinkIO, [x for x in abi.ROOTSINK_FIELDS if x[0] != "qflx_tran_veg_col"],
                              S, ncol, npatch),
            "st": abi.make_io(abi.SoilTempIO, abi.SOILTEMP_FIELDS, S, ncol, npatch),
            "sf": abi.make_io(abi.SoilFluxesIO, abi.SOILFLUXES_FIELDS, S, ncol, npatch),
            "sw": abi.make_io(abi.SoilWaterIO, abi.SOILWATER_FIELDS + abi.SOILWATER_EXTRA, S, ncol),
            "hy": abi.make_io(abi.HydrologyIO, abi.HYDROLOGY_FIELDS, S, ncol),
        }
        self.displa0, self.z0mv0 = S["displa"].copy(), S["z0mv"].copy()
        Bp = C.POINTER(abi.Bounds)
        L.ctsmg_soilevap_resis.argtypes = [Bp, C.c_int32, P32, C.POINTER(abi.SoilResisIO)]
        L.ctsmg_set_soil_resistance.argtypes = [C.POINTER(abi.SoilResistanceParams)]
        L.ctsmg_root_moist_stress.argtypes = [Bp, C.c_int32, P32, C.POINTER(abi.RootMoistIO)]
        L.ctsmg_root_sink.argtypes = [Bp, C.c_int32, P32, C.POINTER(abi.RootSinkIO)]
        L.ctsmg_soiltemperature.argtypes = [Bp, C.c_int32, P32, C.POINTER(abi.SoilTempIO), C.c_double]
        L.ctsmg_soilfluxes.argtypes = [Bp, C.c_int32, P32, C.c_int32, P32, C.POINTER(abi.SoilFluxesIO), C.c_double]
        L.ctsmg_set_soil_water_fractions.argtypes = [Bp, C.c_int32, P32, C.POINTER(abi.SoilWaterIO)]
        L.ctsmg_soilwater.argtypes = [Bp, C.c_int32, P32, C.POINTER(abi.SoilWaterIO), C.c_double]
        L.ctsmg_set_soilhydrology_params.argtypes = [C.POINTER(abi.SoilHydrologyParams)]
        for n in ("ctsmg_saturated_excess_runoff", "ctsmg_perched_water_table", "ctsmg_theta_based_water_table"):
            getattr(L, n).argtypes = [Bp, C.c_int32, P32, C.POINTER(abi.HydrologyIO)]
        for n in ("ctsmg_infiltration_chain", "ctsmg_perched_lateral_flow", "ctsmg_subsurface_lateral_flow"):
            getattr(L, n).argtypes = [Bp, C.c_int32, P32, C.POINTER(abi.HydrologyIO), C.c_double]

    def step(self):
        from ._lib import check
        C, L, S, io, b = self.C, self.L, self.S, self.io, self.C.byref(self.b)
        nc, npt, fc, fp = self.ncol, self.npatch, self.pfc, self.pfp
        S["displa"][:] = self.displa0
        S["z0mv"][:] = self.z0mv0
        S["cgrnds"][:] = 0.0
        S["cgrndl"][:] = 0.0
        check(L.ctsmg_set_soil_resistance(C.byref(self.sres)))
        check(L.ctsmg_soilevap_resis(b, nc, fc, C.byref(io["sr"])))
        check(L.ctsmg_set_canopy_params(C.byref(self.par), C.byref(self.pft)))
        check(L.ctsmg_root_moist_stress(b, npt, fp, C.byref(io["rm"])))
        check(L.ctsmg_canopyfluxes(b, npt, fp, C.byref(io["ci"]), DT))
        check(L.ctsmg_root_sink(b, nc, fc, C.byref(io["rs"])))
        S["tssbef"][:] = S["t_soisno"]
        S["t_h2osfc_bef"][:] = S["t_h2osfc"]
        check(L.ctsmg_soiltemperature(b, nc, fc, C.byref(io["st"]), DT))
        check(L.ctsmg_soilfluxes(b, nc, fc, npt, fp, C.byref(io["sf"]), DT))
        check(L.ctsmg_set_soil_water_fractions(b, nc, fc, C.byref(io["sw"])))
        check(L.ctsmg_set_soilhydrology_params(C.byref(self.hyd)))
        hy = C.byref(io["hy"])
        check(L.ctsmg_saturated_excess_runoff(b, nc, fc, hy))
        check(L.ctsmg_infiltration_chain(b, nc, fc, hy, DT))
        check(L.ctsmg_soilwater(b, nc, fc, C.byref(io["sw"]), DT))
        check(L.ctsmg_perched_water_table(b, nc, fc, hy))
        check(L.ctsmg_theta_based_water_table(b, nc, fc, hy))
        check(L.ctsmg_perched_lateral_flow(b, nc, fc, hy, DT))
        check(L.ctsmg_subsurface_lateral_flow(b, nc, fc, hy, DT))
        inputs.refresh_h2osoi_vol(S)
