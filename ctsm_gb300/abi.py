"""ctypes mirror of include/ctsm_gpu.h and the field manifest of the soil path.

The manifest records, for every derived-type component the C-ABI carries, its
level kind (which fixes its Fortran lower bound and level count), its element
type and whether the call reads it, writes it, or both.  The same manifest
drives the host state container, the device buffers of the batched engine and
the algorithmic-byte count used for the roofline.
"""
import ctypes as C

NLEVSNO = 12
NLEVSOI = 20
NLEVGRND = 25

# level kind -> (lower bound, number of levels); the C-ABI stores element
# (c, j) at base[(c - begc) + (j - lb) * ld]  (src/main/ColumnType.F90:137-155)
LEVELS = {
    "C": (None, 1),                       # scalar per column (1-D)
    "P": (None, 1),                       # scalar per patch (1-D)
    "SS": (-NLEVSNO + 1, NLEVSNO + NLEVGRND),
    "ZI": (-NLEVSNO, NLEVSNO + NLEVGRND + 1),
    "G": (1, NLEVGRND),
    "S": (1, NLEVSOI),
    "SN": (-NLEVSNO + 1, NLEVSNO),
    "PL": (-NLEVSNO + 1, NLEVSNO + 1),    # patch, snow levels + top soil
    "GR": (None, 1),                      # scalar per gridcell (1-D)
    "PG": (1, NLEVGRND),                  # patch, soil + bedrock levels
}

F64, I32 = "f8", "i4"

# (name, kind, dtype, use) in the order of the C structs; use: in / out / inout
SOILWATER_FIELDS = [
    ("z", "SS", F64, "in"), ("zi", "ZI", F64, "in"), ("dz", "SS", F64, "in"),
    ("zwt", "C", F64, "in"), ("qcharge", "C", F64, "out"), ("icefrac", "G", F64, "out"),
    ("qin", "S", F64, "out"), ("qout", "S", F64, "out"),
    ("smpmin", "C", F64, "in"), ("watsat", "G", F64, "in"), ("hksat", "G", F64, "in"),
    ("bsw", "G", F64, "in"), ("sucsat", "G", F64, "in"),
    ("smp_l", "G", F64, "out"), ("hk_l", "G", F64, "out"),
    ("h2osoi_ice", "SS", F64, "in"), ("h2osoi_liq", "SS", F64, "inout"),
    ("h2osoi_vol", "G", F64, "in"),
    ("qflx_deficit", "C", F64, "out"), ("qflx_infl", "C", F64, "in"),
    ("qflx_rootsoi", "S", F64, "in"),
    ("t_soisno", "SS", F64, "in"),
]

# components only the moisture form or the flexibleCN fix use (NULL otherwise)
SOILWATER_EXTRA = [
    ("nbedrock", "C", I32, "in"), ("eff_porosity", "G", F64, "in"), ("num_substeps", "C", F64, "out"),
    ("wa", "C", F64, "inout"),
]

SOILTEMP_FIELDS = [
    ("snl", "C", I32, "in"), ("nbedrock", "C", I32, "in"),
    ("z", "SS", F64, "in"), ("zi", "ZI", F64, "in"), ("dz", "SS", F64, "in"),
    ("col_patchi", "C", I32, "in"), ("col_npatches", "C", I32, "in"),
    ("wtcol", "P", F64, "in"), ("frac_veg_nosno", "P", I32, "in"),
    ("forc_lwrad", "C", F64, "in"), ("sabg", "P", F64, "in"), ("sabg_soil", "P", F64, "in"),
    ("sabg_snow", "P", F64, "in"), ("sabg_lyr", "PL", F64, "in"), ("sabg_chk", "P", F64, "out"),
    ("htvp", "C", F64, "in"), ("cgrnd", "P", F64, "in"), ("dlrad", "P", F64, "in"),
    ("eflx_sh_grnd", "P", F64, "in"), ("eflx_sh_snow", "P", F64, "in"),
    ("eflx_sh_soil", "P", F64, "in"), ("eflx_sh_h2osfc", "P", F64, "in"),
    ("qflx_evap_soi", "P", F64, "in"), ("qflx_ev_snow", "P", F64, "in"),
    ("qflx_ev_soil", "P", F64, "in"), ("qflx_ev_h2osfc", "P", F64, "in"),
    ("eflx_bot", "C", F64, "in"),
    ("eflx_gnet", "P", F64, "out"), ("dgnetdT", "P", F64, "out"),
    ("eflx_fgr12", "C", F64, "out"), ("eflx_fgr", "G", F64, "out"),
    ("eflx_snomelt", "C", F64, "out"), ("eflx_h2osfc_to_snow", "C", F64, "out"),
    ("emg", "C", F64, "in"), ("t_soisno", "SS", F64, "inout"), ("t_h2osfc", "C", F64, "inout"),
    ("t_grnd", "C", F64, "inout"), ("fact", "SS", F64, "out"), ("c_h2osfc", "C", F64, "out"),
    ("xmf", "C", F64, "out"), ("xmf_h2osfc", "C", F64, "out"), ("imelt", "SS", I32, "out"),
    ("watsat", "G", F64, "in"), ("bsw", "G", F64, "in"), ("sucsat", "G", F64, "in"),
    ("tkmg", "G", F64, "in"), ("tkdry", "G", F64, "in"), ("csol", "G", F64, "in"),
    ("thk", "SS", F64, "out"),
    ("h2osoi_liq", "SS", F64, "inout"), ("h2osoi_ice", "SS", F64, "inout"),
    ("h2osfc", "C", F64, "inout"), ("h2osno_no_layers", "C", F64, "inout"),
    ("int_snow", "C", F64, "inout"), ("snow_depth", "C", F64, "inout"),
    ("snomelt_accum", "C", F64, "inout"),
    ("frac_sno_eff", "C", F64, "in"), ("frac_h2osfc", "C", F64, "in"),
    ("bw", "SN", F64, "out"), ("qflx_snomelt", "C", F64, "out"), ("qflx_snofrz", "C", F64, "out"),
    ("qflx_snow_drain", "C", F64, "out"), ("qflx_snomelt_lyr", "SN", F64, "out"),
    ("qflx_snofrz_lyr", "SN", F64, "out"), ("qflx_h2osfc_to_ice", "C", F64, "out"),
]


_P_IN = ["elai", "esai", "htop", "emv", "fwet", "fdry", "laisun", "laisha", "btran", "sabv", "thm", "t_a10",
         "parsun_z", "parsha_z", "vcmaxcintsun", "vcmaxcintsha"]
_P_INOUT = ["displa", "z0mv", "t_veg", "liqcan", "snocan", "cgrnds", "cgrndl"]
_P_OUT = ["z0hv", "z0qv", "forc_hgt_u_patch", "forc_hgt_t_patch", "forc_hgt_q_patch", "taf", "qaf", "ustar", "um",
          "obu", "zeta", "ram1", "rah1", "raw1", "rah2", "raw2", "rb1", "uaf", "vpd", "rhaf",
          "eflx_sh_veg", "qflx_evap_veg", "qflx_tran_veg", "eflx_sh_grnd", "eflx_sh_snow", "eflx_sh_soil",
          "eflx_sh_h2osfc", "qflx_evap_soi", "qflx_ev_snow", "qflx_ev_soil", "qflx_ev_h2osfc",
          "t_ref2m", "q_ref2m", "rh_ref2m", "vpd_ref2m", "dlrad", "ulrad", "t_skin", "cgrnd", "taux", "tauy",
          "err_canopy", "rssun", "rssha", "psnsun", "psnsha", "lmrsun", "lmrsha", "cisun", "cisha", "gs_mol_sun",
          "gs_mol_sha", "rh_leaf", "vpd_can", "u10_clm", "u10", "fv", "vds", "fm"]
CANOPY_FIELDS = (
    [("itype", "P", I32, "in"), ("patch_column", "P", I32, "in"), ("patch_gridcell", "P", I32, "in")] +
    [(n, "GR", F64, "in") for n in ("forc_u", "forc_v", "forc_hgt_u", "forc_hgt_t", "forc_hgt_q", "forc_pco2",
                                      "forc_po2", "dayl", "max_dayl")] +
    [("snl", "C", I32, "in")] +
    [(n, "C", F64, "in") for n in ("forc_pbot", "forc_th", "forc_q", "forc_rho", "forc_lwrad", "thv", "t_grnd",
                                     "qg", "qg_snow", "qg_soil", "qg_h2osfc", "dqgdT", "emg", "htvp", "z0mg",
                                     "snow_depth", "frac_sno_eff", "frac_h2osfc", "soilresis", "t_h2osfc")] +
    [("t_soisno", "SS", F64, "in"), ("frac_veg_nosno", "P", I32, "in")] +
    [(n, "P", F64, "in") for n in _P_IN] +
    [(n, "P", F64, "inout") for n in _P_INOUT] +
    [(n, "P", F64, "out") for n in _P_OUT] +
    [("num_iter", "P", I32, "out")])


# SoilFluxes (src/biogeophys/SoilFluxesMod.F90:36-518), natural-vegetation
# columns and patches; tssbef / t_h2osfc_bef are the temperatures saved before
# SoilTemperature.
SOILFLUXES_FIELDS = [
    ("snl", "C", I32, "in"), ("col_patchi", "C", I32, "in"), ("col_npatches", "C", I32, "in"),
    ("frac_sno_eff", "C", F64, "in"), ("frac_h2osfc", "C", F64, "in"), ("t_grnd", "C", F64, "in"),
    ("t_h2osfc", "C", F64, "in"), ("t_h2osfc_bef", "C", F64, "in"), ("c_h2osfc", "C", F64, "in"),
    ("emg", "C", F64, "in"), ("forc_lwrad", "C", F64, "in"), ("htvp", "C", F64, "in"),
    ("xmf", "C", F64, "in"), ("xmf_h2osfc", "C", F64, "in"), ("eflx_h2osfc_to_snow", "C", F64, "in"),
    ("t_soisno", "SS", F64, "in"), ("tssbef", "SS", F64, "in"), ("fact", "SS", F64, "in"),
    ("h2osoi_liq", "SS", F64, "in"), ("h2osoi_ice", "SS", F64, "in"),
    ("errsoi_col", "C", F64, "out"),
    ("patch_column", "P", I32, "in"), ("frac_veg_nosno", "P", I32, "in"), ("wtcol", "P", F64, "in"),
    ("cgrnds", "P", F64, "in"), ("cgrndl", "P", F64, "in"), ("sabg_soil", "P", F64, "in"),
    ("sabg_snow", "P", F64, "in"), ("dlrad", "P", F64, "in"), ("ulrad", "P", F64, "in"),
    ("eflx_sh_veg", "P", F64, "in"), ("qflx_evap_veg", "P", F64, "in"), ("qflx_tran_veg", "P", F64, "in"),
    ("eflx_sh_grnd", "P", F64, "inout"), ("qflx_evap_soi", "P", F64, "inout"),
    ("qflx_ev_snow", "P", F64, "inout"), ("qflx_ev_soil", "P", F64, "inout"), ("qflx_ev_h2osfc", "P", F64, "inout"),
    ("qflx_liqevap_from_top_layer", "P", F64, "out"), ("qflx_solidevap_from_top_layer", "P", F64, "out"),
    ("qflx_soliddew_to_top_layer", "P", F64, "out"), ("qflx_liqdew_to_top_layer", "P", F64, "out"),
    ("eflx_soil_grnd", "P", F64, "out"), ("eflx_sh_tot", "P", F64, "out"), ("qflx_evap_tot", "P", F64, "out"),
    ("eflx_lh_tot", "P", F64, "out"), ("qflx_evap_can", "P", F64, "out"), ("eflx_lh_vege", "P", F64, "out"),
    ("eflx_lh_vegt", "P", F64, "out"), ("eflx_lh_grnd", "P", F64, "out"), ("eflx_lwrad_out", "P", F64, "out"),
    ("eflx_lwrad_net", "P", F64, "out"), ("errsoi_patch", "P", F64, "out"), ("t_skin", "P", F64, "inout"),
]


# Root moisture stress (SoilMoistStressMod.F90:70-217, 312-435) as run at the
# start of CanopyFluxes (CanopyFluxesMod.F90:709, 833-895).
ROOTMOIST_FIELDS = [
    ("h2osoi_liq", "SS", F64, "in"), ("h2osoi_ice", "SS", F64, "in"), ("dz", "SS", F64, "in"),
    ("t_soisno", "SS", F64, "in"), ("watsat", "G", F64, "in"), ("sucsat", "G", F64, "in"), ("bsw", "G", F64, "in"),
    ("eff_porosity", "G", F64, "out"), ("h2osoi_liqvol", "G", F64, "out"),
    ("patch_column", "P", I32, "in"), ("itype", "P", I32, "in"), ("rootfr", "PG", F64, "in"),
    ("btran", "P", F64, "out"), ("rootr", "PG", F64, "out"), ("rresis", "PG", F64, "inout"),
]


# BareGroundFluxes (BareGroundFluxesMod.F90:73-545), in the order of
# ctsmg_baregrnd_io after ldp, ldc, ldg, begg
BAREGRND_FIELDS = (
    [("patch_column", "P", I32, "in"), ("patch_gridcell", "P", I32, "in")] +
    [(n, "GR", F64, "in") for n in ("forc_u", "forc_v", "forc_hgt_u", "forc_hgt_t", "forc_hgt_q")] +
    [("snl", "C", I32, "in")] +
    [(n, "C", F64, "in") for n in ("forc_t", "forc_pbot", "forc_q", "forc_th", "forc_rho", "thv", "t_grnd", "qg",
                                     "qg_snow", "qg_soil", "qg_h2osfc", "dqgdT", "htvp", "z0mg", "soilresis",
                                     "soilbeta", "t_h2osfc")] +
    [("t_soisno", "SS", F64, "in"), ("z0hg", "C", F64, "inout"), ("z0qg", "C", F64, "inout"),
     ("thm", "P", F64, "in")] +
    [(n, "P", F64, "inout") for n in ("forc_hgt_u_patch", "forc_hgt_t_patch", "forc_hgt_q_patch")] +
    [(n, "P", F64, "out") for n in (
        "btran", "t_veg", "rssun", "rssha", "displa", "z0mv", "z0hv", "z0qv", "dlrad", "ulrad", "dhsdt_canopy",
        "eflx_sh_stem", "z0mg_patch", "z0hg_patch", "z0qg_patch", "zeta", "obu", "ram1", "cgrnds", "cgrndl", "cgrnd",
        "taux", "tauy", "eflx_sh_grnd", "eflx_sh_tot", "eflx_sh_snow", "eflx_sh_soil", "eflx_sh_h2osfc",
        "qflx_tran_veg", "qflx_evap_veg", "qflx_evap_soi", "qflx_evap_tot", "qflx_ev_snow", "qflx_ev_soil",
        "qflx_ev_h2osfc", "t_ref2m", "q_ref2m", "rh_ref2m", "kbm1", "u10_clm", "u10", "va", "vds", "fv", "fm")] +
    [("num_iter", "P", I32, "out"), ("rootr", "PG", F64, "out"), ("rresis", "PG", F64, "out")])

# hydrology neighbours of SoilWater (ctsmg_hydrology_io order after ldc)
HYDROLOGY_FIELDS = [
    ("nbedrock", "C", I32, "in"), ("z", "SS", F64, "in"), ("zi", "ZI", F64, "in"), ("dz", "SS", F64, "in"),
    ("t_soisno", "SS", F64, "in"), ("h2osoi_liq", "SS", F64, "inout"), ("h2osoi_ice", "SS", F64, "inout"),
    ("h2osoi_vol", "G", F64, "inout"), ("h2osfc", "C", F64, "inout"), ("zwt", "C", F64, "inout"),
    ("zwt_perched", "C", F64, "inout"), ("frost_table", "C", F64, "inout"), ("icefrac", "G", F64, "out"),
    ("watsat", "G", F64, "in"), ("hksat", "G", F64, "in"), ("bsw", "G", F64, "in"), ("sucsat", "G", F64, "in"),
    ("eff_porosity", "G", F64, "in"), ("topo_slope", "C", F64, "in"), ("wtfact", "C", F64, "in"),
    ("qflx_rain_plus_snomelt", "C", F64, "in"), ("qflx_snwcp_liq", "C", F64, "in"),
    ("fsat", "C", F64, "out"), ("fcov", "C", F64, "out"), ("qflx_sat_excess_surf", "C", F64, "out"),
    ("qflx_drain_perched", "C", F64, "out"), ("qflx_latflow_out", "C", F64, "out"),
    ("qflx_latflow_in", "C", F64, "out"), ("qflx_rsub_sat", "C", F64, "out"), ("qflx_drain", "C", F64, "out"),
    ("qflx_qrgwl", "C", F64, "out"), ("qflx_ice_runoff_xs", "C", F64, "out"),
    ("snl", "C", I32, "in"),
] + [(n, "C", F64, "in") for n in ("frac_sno_eff", "frac_h2osfc", "frac_h2osfc_nosnow", "h2osfc_thresh",
                                    "qflx_snow_h2osfc", "qflx_floodc", "qflx_ev_soil_col",
                                    "qflx_liqevap_from_top_layer_col", "qflx_ev_h2osfc_col")] + \
    [(n, "C", F64, "out") for n in ("qflx_top_soil", "qflx_in_soil", "qflx_top_soil_to_h2osfc", "qinmax",
                                     "qflx_infl_excess", "qflx_in_soil_limited", "qflx_in_h2osfc",
                                     "qflx_infl_excess_surf", "qflx_h2osfc_surf", "qflx_h2osfc_drain", "qflx_infl")] + \
    [("wa", "C", F64, "inout"), ("qcharge", "C", F64, "in"), ("hkdepth", "C", F64, "in")]

# calc_soilevap_resis (sl_14 uses dsl/soilresis, leepielke_1992 soilbeta)
SOILRESIS_FIELDS = [
    ("dz", "SS", F64, "in"), ("t_soisno", "SS", F64, "in"), ("h2osoi_liq", "SS", F64, "in"),
    ("h2osoi_ice", "SS", F64, "in"), ("watsat", "G", F64, "in"), ("bsw", "G", F64, "in"), ("sucsat", "G", F64, "in"),
    ("watfc", "G", F64, "in"), ("frac_sno", "C", F64, "in"), ("frac_h2osfc", "C", F64, "in"),
    ("dsl", "C", F64, "out"), ("soilresis", "C", F64, "out"), ("soilbeta", "C", F64, "out"),
]


def _ptr_type(dtype):
    return C.POINTER(C.c_double) if dtype == F64 else C.POINTER(C.c_int32)


class Bounds(C.Structure):
    _fields_ = [("begc", C.c_int32), ("endc", C.c_int32), ("begp", C.c_int32), ("endp", C.c_int32)]


class Options(C.Structure):
    _fields_ = [("soilwater_movement_method", C.c_int32), ("snow_thermal_cond_method", C.c_int32),
                ("itmax_canopy_fluxes", C.c_int32), ("stomatalcond_method", C.c_int32),
                ("nlevsno", C.c_int32), ("nlevsoi", C.c_int32), ("nlevgrnd", C.c_int32)]


class SoilWaterParams(C.Structure):
    _fields_ = [("e_ice", C.c_double)]


class SoilWaterIO(C.Structure):
    _fields_ = [("ldc", C.c_int32)] + [(n, _ptr_type(t)) for (n, _, t, _) in SOILWATER_FIELDS + SOILWATER_EXTRA]


class BareGrndIO(C.Structure):
    _fields_ = [("ldp", C.c_int32), ("ldc", C.c_int32), ("ldg", C.c_int32), ("begg", C.c_int32)] + \
               [(n, _ptr_type(t)) for (n, _, t, _) in BAREGRND_FIELDS]


class HydrologyIO(C.Structure):
    _fields_ = [("ldc", C.c_int32)] + [(n, _ptr_type(t)) for (n, _, t, _) in HYDROLOGY_FIELDS]


class SoilHydrologyParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("aq_sp_yield_min", "n_baseflow", "baseflow_scalar",
                                           "perched_baseflow_scalar", "e_ice", "fff", "pc", "mu")] + \
               [("h2osfcflag", C.c_int32)]


class SoilResisIO(C.Structure):
    _fields_ = [("ldc", C.c_int32)] + [(n, _ptr_type(t)) for (n, _, t, _) in SOILRESIS_FIELDS]


class SoilResistanceParams(C.Structure):
    _fields_ = [("soil_resis_method", C.c_int32), ("d_max", C.c_double), ("frac_sat_soil_dsl_init", C.c_double)]


class SoilWaterMovementNml(C.Structure):
    _fields_ = [("soilwater_movement_method", C.c_int32), ("upper_boundary_condition", C.c_int32),
                ("lower_boundary_condition", C.c_int32), ("flux_calculation", C.c_int32),
                ("use_flexibleCN", C.c_int32), ("use_bedrock", C.c_int32), ("dtmin", C.c_double),
                ("verySmall", C.c_double), ("xTolerUpper", C.c_double), ("xTolerLower", C.c_double)]


def soilwater_movement_nml(method=1, upper=1, lower=None, flux_calculation=1, use_flexibleCN=0, use_bedrock=1,
                           dtmin=60.0, verySmall=1e-8, xTolerUpper=1e-1, xTolerLower=1e-2):
    """The namelist with the reference's defaults (namelist_defaults_ctsm.xml:471-488)."""
    if lower is None:
        lower = 4 if method == 0 else 2
    return SoilWaterMovementNml(method, upper, lower, flux_calculation, use_flexibleCN, use_bedrock, dtmin,
                                verySmall, xTolerUpper, xTolerLower)


ROOTSINK_FIELDS = [
    ("col_patchi", "C", I32, "in"), ("col_npatches", "C", I32, "in"), ("wtcol", "P", F64, "in"),
    ("qflx_tran_veg", "P", F64, "in"), ("qflx_tran_veg_col", "C", F64, "in"), ("rootr", "PG", F64, "in"),
    ("rootr_col", "G", F64, "out"), ("qflx_rootsoi", "S", F64, "out"),
]


class RootSinkIO(C.Structure):
    _fields_ = [("ldc", C.c_int32), ("ldp", C.c_int32)] + \
               [(n, _ptr_type(t)) for (n, _, t, _) in ROOTSINK_FIELDS]


class RootMoistIO(C.Structure):
    _fields_ = [("ldc", C.c_int32), ("ldp", C.c_int32)] + \
               [(n, _ptr_type(t)) for (n, _, t, _) in ROOTMOIST_FIELDS]


class SoilFluxesIO(C.Structure):
    _fields_ = [("ldc", C.c_int32), ("ldp", C.c_int32)] + \
               [(n, _ptr_type(t)) for (n, _, t, _) in SOILFLUXES_FIELDS]


class SoilTempIO(C.Structure):
    _fields_ = [("ldc", C.c_int32), ("ldp", C.c_int32)] + \
               [(n, _ptr_type(t)) for (n, _, t, _) in SOILTEMP_FIELDS]


class CanopyParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "lai_dl", "z_dl", "a_coef", "a_exp", "csoilc", "cv", "wind_min", "zetamaxstable",
        "kc25_coef", "ko25_coef", "cp25_yr2000", "kcha", "koha", "cpha",
        "vcmaxha", "jmaxha", "tpuha", "lmrha", "vcmaxhd", "jmaxhd", "tpuhd", "lmrhd", "lmrse",
        "vcmaxse_sf", "jmaxse_sf", "tpuse_sf", "jmax25top_sf",
        "fnr", "act25", "theta_psii", "theta_ip", "tpu25ratio", "kp25ratio", "fnps", "leaf_mr_vcm")] + \
        [("light_inhibit", C.c_int32)]


MAX_PFT = 80


class Pftcon(C.Structure):
    _fields_ = [("npft", C.c_int32)] + [(n, C.c_double * MAX_PFT) for n in (
        "c3psn", "slatop", "leafcn", "flnr", "fnitr", "dleaf", "medlynslope", "medlynintercept", "theta_cj",
        "mbbopt", "smpso", "smpsc")]


class CanopyIO(C.Structure):
    _fields_ = [("ldp", C.c_int32), ("ldc", C.c_int32), ("ldg", C.c_int32), ("begg", C.c_int32)] + \
               [(n, _ptr_type(t)) for (n, _, t, _) in CANOPY_FIELDS]


def field_shape(kind, ncol, npatch, ngrid=None):
    """numpy shape (levels, columns-or-patches) of a manifest field."""
    if kind == "GR":
        return (ngrid if ngrid is not None else ncol,)
    n = npatch if kind in ("P", "PL", "PS", "PG") else ncol
    nlev = LEVELS[kind][1]
    return (n,) if kind in ("C", "P") else (nlev, n)


def make_io(cls, fields, arrays, ldc, ldp=None, ldg=None, begg=1):
    """Fill a ctypes io struct with pointers into the numpy arrays of `arrays`."""
    io = cls()
    io.ldc = ldc
    if ldp is not None:
        io.ldp = ldp
    if ldg is not None:
        io.ldg = ldg
        io.begg = begg
    for (n, _, t, _) in fields:
        a = arrays[n]
        assert a.flags.c_contiguous, n
        setattr(io, n, a.ctypes.data_as(_ptr_type(t)))
    return io
