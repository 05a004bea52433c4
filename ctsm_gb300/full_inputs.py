"""Seeded inputs for the full soil + canopy step (CanopyFluxes, SoilTemperature,
SoilWater) and for the perturbed-parameter ensemble.

One consistent state: the columns come from inputs.soil_columns (snow, uneven
bedrock, 1-4 patches per column, every ground flux drawn), their patches
from canopy_inputs.canopy_patches, and every component the two share
(snl, t_soisno, t_grnd, t_h2osfc, frac_sno_eff, frac_h2osfc, snow_depth, emg,
htvp, forc_lwrad, frac_veg_nosno, the patch/column maps) is taken from the
soil state.  The air temperature of a column is its ground temperature plus
U(-5,5) K; the ground humidities follow SurfaceHumidityMod.F90:185-216 (qg_snow =
qg_soil on snow-free columns, qg their fraction-weighted mix).  Root fractions of every patch follow the fixed profile
dz_j exp(-3 z_j) (normalised) that the plain workloads use for the sink.

Ensemble members perturb 8 parameters by a factor drawn log-uniformly in
[0.5, 1.5] (baseflow_scalar, fff, medlynslope, medlynintercept, jmaxb1, kmax,
om_frac_sf, d_max).  medlynslope and medlynintercept enter Photosynthesis (per
patch) and om_frac_sf the soil-property preparation.  With clm5=True the
members run the CLM5-default step, where three more act per column:
baseflow_scalar in SubsurfaceLateralFlow (SoilHydrologyMod.F90:2336), fff in
SaturatedExcessRunoff (SaturatedExcessRunoffMod.F90:352) and d_max in the
sl_14 soil resistance (SurfaceResistanceMod.F90:404).  jmaxb1 belongs to LUNA
(LunaMod.F90:419) and kmax to the plant-hydraulic-stress photosynthesis
(PhotosynthesisMod.F90:846), both outside the path: they are stored per
member without effect.
"""
import numpy as np

from . import abi, inputs, canopy_inputs

ENSEMBLE_PARAMS = ("baseflow_scalar", "fff", "medlynslope", "medlynintercept", "jmaxb1", "kmax", "om_frac_sf",
                   "d_max")
# defaults the member factors scale (the parameter-file values, absent here,
# are builder's choices: ctsm_gb300.soil.set_soilhydrology_params /
# set_soil_resistance use the same)
BASEFLOW_SCALAR, FFF, D_MAX = 1.0e-2, 0.5, 15.0


def full_state(ncol, seed=0, npatch_max=4, om_frac_sf=1.0, rng=None):
    """Returns (A, npatch, ngrid, rootr): A holds every soil and canopy
    component; rootr is (nlevsoi, npatch)."""
    r = rng if rng is not None else np.random.Generator(np.random.Philox(seed))
    A, npatch = inputs.soil_columns(ncol, snow=True, nbedrock=(3, 20), forcing="full", npatch_max=npatch_max,
                                    rng=r)
    if om_frac_sf != 1.0:
        _reprep_soil(A, r, om_frac_sf)
    Cn, _, _, _ = canopy_inputs.canopy_patches(npatch, npatch_max=1, rng=r)
    ngrid = ncol
    pcol = np.repeat(np.arange(ncol), A["col_npatches"])
    # patch -> column / gridcell maps from the soil state
    Cn["patch_column"] = (pcol + 1).astype(np.int32)
    Cn["patch_gridcell"] = (pcol + 1).astype(np.int32)
    # columns: the canopy generator drew one column per patch; draw the
    # atmosphere per column again, tied to the ground temperature
    tg = A["t_grnd"]
    forc_t = tg + r.uniform(-5.0, 5.0, ncol)
    pbot = r.uniform(86000.0, 101325.0, ncol)
    qs, _, _ = canopy_inputs.qsat(forc_t, pbot)
    rh = r.uniform(0.10, 1.00, ncol)
    forc_q = rh * qs
    forc_th = forc_t * (100000.0 / pbot) ** (canopy_inputs.RAIR / canopy_inputs.CPAIR)
    e = forc_q * pbot / (0.622 + 0.378 * forc_q)
    col = dict(forc_pbot=pbot, forc_q=forc_q, forc_th=forc_th,
               forc_rho=(pbot - 0.378 * e) / (canopy_inputs.RAIR * forc_t),
               thv=forc_th * (1.0 + 0.61 * forc_q))
    # ground humidities by the rules of SurfaceHumidityMod.F90:185-216
    LS = -abi.NLEVSNO + 1
    snl = A["snl"]
    t1 = A["t_soisno"][1 - LS]
    ttop = A["t_soisno"][snl + 1 - LS, np.arange(ncol)]
    fsno, fh2o = A["frac_sno_eff"], A["frac_h2osfc"]
    q_soil, _, dq_soil = canopy_inputs.qsat(t1, pbot)
    q_snow, _, dq_snow = canopy_inputs.qsat(ttop, pbot)
    hr = r.uniform(0.5, 1.0, ncol)
    qg_soil = hr * q_soil
    qg_snow = np.where(snl < 0, q_snow, qg_soil)
    dqgdT = np.where(snl < 0, fsno * dq_snow + (1.0 - fsno - fh2o) * hr * dq_soil, (1.0 - fh2o) * hr * dq_soil)
    qg_h2osfc = qg_soil
    qg = fsno * qg_snow + (1.0 - fsno - fh2o) * qg_soil + fh2o * qg_h2osfc
    col.update(qg=qg, qg_snow=qg_snow, qg_soil=qg_soil, qg_h2osfc=qg_h2osfc, dqgdT=dqgdT,
               z0mg=np.full(ncol, 0.01), soilresis=r.uniform(50.0, 5000.0, ncol))
    grid = dict(forc_u=r.uniform(0.5, 20.0, ngrid), forc_v=np.zeros(ngrid), forc_hgt_u=np.full(ngrid, 30.0),
                forc_hgt_t=np.full(ngrid, 30.0), forc_hgt_q=np.full(ngrid, 30.0), forc_pco2=400.e-6 * pbot,
                forc_po2=0.209 * pbot, dayl=r.uniform(28800.0, 57600.0, ngrid), max_dayl=np.full(ngrid, 57600.0))
    col["forc_t"] = forc_t
    for k, v in list(col.items()) + list(grid.items()):
        A[k] = np.ascontiguousarray(v)
    A["thm"] = forc_t[pcol] + 0.0098 * 30.0
    A["t_a10"] = forc_t[pcol] + r.uniform(-3.0, 3.0, npatch)
    A["t_veg"] = forc_t[pcol] + r.uniform(-2.0, 2.0, npatch)
    A["snocan"] = np.where(A["t_veg"] < canopy_inputs.TFRZ, Cn["snocan"], 0.0)
    # remaining canopy components (vegetation, radiation, outputs)
    for (n, kind, dt, use) in abi.CANOPY_FIELDS:
        if n not in A:
            A[n] = Cn[n]
    A["frac_veg_nosno"][:] = 1
    A["eflx_bot"][:] = 0.0            # no heat flux from beneath the column, as for CTSM's soil columns
    # absorbed ground solar consistent with the soil's sabg_lyr (sum over layers)
    dzs, zs, _ = inputs.layer_structure_20sl()
    prof = np.array([dzs[j] * np.exp(-3.0 * zs[j]) for j in range(abi.NLEVSOI)])
    prof = prof / prof.sum()
    rootr = np.ascontiguousarray(np.repeat(prof[:, None], npatch, axis=1))
    return A, npatch, ngrid, rootr


def _reprep_soil(A, r, om_frac_sf):
    """Soil properties with the organic-matter scale factor om_frac_sf
    (SoilStateInitTimeConstMod.F90:452: om_frac = min(om_frac_sf*om/organic_max, 1))."""
    ncol = A["zwt"].shape[0]
    sand = r.uniform(5.0, 80.0, ncol)
    clay = np.minimum(r.uniform(5.0, 85.0, ncol), 95.0 - sand)
    om = np.minimum(r.uniform(0.0, 130.0, ncol) * om_frac_sf, inputs.ORGANIC_MAX)
    _, zs, _ = inputs.layer_structure_20sl()
    props = inputs.pedotransfer(sand, clay, om, zs)
    for k in ("watsat", "bsw", "sucsat", "hksat", "tkmg", "tkdry", "csol"):
        A[k][:] = props[k]


def ensemble(nmembers, seed=0, cols=(512, 8192), npatch_max=4, clm5=False):
    """Pack `nmembers` members (column counts U{cols}) into one state.
    Returns (A, npatch, ngrid, rootr, member_of_column, params) with params a
    dict name -> (nmembers,) factors and per-patch Medlyn arrays in A.  With
    clm5=True A also holds the components of the CLM5-default step (SoilFluxes,
    root moisture stress, soil resistance, the default hydrology) and the
    members' per-column baseflow_scalar_c, fff_c and d_max_c."""
    r = np.random.Generator(np.random.Philox(seed))
    factors = {k: np.exp(r.uniform(np.log(0.5), np.log(1.5), nmembers)) for k in ENSEMBLE_PARAMS}
    ncols = r.integers(cols[0], cols[1] + 1, nmembers)
    parts = []
    for m in range(nmembers):
        rm = np.random.Generator(np.random.Philox(seed * 1000003 + m + 1))
        parts.append(full_state(int(ncols[m]), npatch_max=npatch_max, om_frac_sf=float(factors["om_frac_sf"][m]),
                                rng=rm))
    A, npatch, ngrid, rootr = concat(parts)
    member_col = np.repeat(np.arange(nmembers), ncols).astype(np.int32)
    member_patch = np.repeat(np.arange(nmembers), [p[1] for p in parts]).astype(np.int32)
    pft = canopy_inputs.DEFAULT_PFT
    it = A["itype"]
    base_slope = np.array([row[6] for row in pft])[it]
    base_int = np.array([row[7] for row in pft])[it]
    A["medlynslope_p"] = np.ascontiguousarray(base_slope * factors["medlynslope"][member_patch])
    A["medlynintercept_p"] = np.ascontiguousarray(base_int * factors["medlynintercept"][member_patch])
    if clm5:
        rc = np.random.Generator(np.random.Philox(seed * 1000003 + nmembers + 7))
        add_soilfluxes_fields(A, npatch, ngrid)
        add_rootmoist_fields(A, npatch, rootr, rng=rc)
        add_soilresis_fields(A)
        add_hydrology_fields(A, rc)
        A["baseflow_scalar_c"] = np.ascontiguousarray(BASEFLOW_SCALAR * factors["baseflow_scalar"][member_col])
        A["fff_c"] = np.ascontiguousarray(FFF * factors["fff"][member_col])
        A["d_max_c"] = np.ascontiguousarray(D_MAX * factors["d_max"][member_col])
        A["rootr_col"] = np.zeros((abi.NLEVGRND, A["zwt"].shape[0]))     # written by the root sink
    return A, npatch, ngrid, rootr, member_col, factors


def concat(parts):
    """Concatenate full states along columns / patches / gridcells, fixing the
    1-based index maps."""
    out = {}
    ncol_off = npat_off = 0
    pieces = {}
    for (A, npatch, ngrid, rootr) in parts:
        ncol = A["zwt"].shape[0]
        B = dict(A)
        B["col_patchi"] = A["col_patchi"] + npat_off
        B["patch_column"] = A["patch_column"] + ncol_off
        B["patch_gridcell"] = A["patch_gridcell"] + ncol_off
        B["_rootr"] = rootr
        for k, v in B.items():
            pieces.setdefault(k, []).append(v)
        ncol_off += ncol
        npat_off += npatch
    for k, vs in pieces.items():
        out[k] = np.ascontiguousarray(np.concatenate(vs, axis=-1))
    rootr = out.pop("_rootr")
    return out, npat_off, ncol_off, rootr


def add_soilfluxes_fields(A, npatch, ngrid):
    """Zero-filled arrays for the SoilFluxes components a full state lacks
    (tssbef / t_h2osfc_bef are written by the step before SoilTemperature)."""
    ncol = A["zwt"].shape[0]
    for (n, kind, t, u) in abi.SOILFLUXES_FIELDS:
        if n not in A:
            A[n] = np.zeros(abi.field_shape(kind, ncol, npatch, ngrid), dtype=np.dtype(t))
    return A


def snow_free(A):
    """Workload columns with their snow layers taken away (snl = 0): melted
    snow layers are removed only by SnowHydrology, outside the path, and a
    layer that has melted but stays a layer heats without bound in the
    reference's arithmetic (the oracle shows it within days)."""
    LS = -abi.NLEVSNO + 1
    A["snl"][:] = 0
    for j in range(LS, 1):
        A["h2osoi_liq"][j - LS] = 0.0
        A["h2osoi_ice"][j - LS] = 0.0
        A["dz"][j - LS] = 0.0
    for k in ("frac_sno_eff", "frac_sno", "snow_depth", "h2osno_no_layers"):
        if k in A:
            A[k][:] = 0.0
    return A


def add_rootmoist_fields(A, npatch, rootr, rng=None):
    """Root fractions (levels 1..nlevgrnd, zero below nlevsoi as
    RootBiophysMod leaves them) and zero-filled stress outputs.  rootfr is the
    state's nlevsoi root profile, jittered per patch when rng is given."""
    ncol = A["zwt"].shape[0]
    fr = np.zeros((abi.NLEVGRND, npatch))
    fr[:abi.NLEVSOI] = rootr[:, :npatch]
    if rng is not None:
        fr[:abi.NLEVSOI] *= rng.uniform(0.5, 1.5, (abi.NLEVSOI, npatch))
        fr /= fr.sum(axis=0, keepdims=True)
    A["rootfr"] = np.ascontiguousarray(fr)
    for (n, kind, t, u) in abi.ROOTMOIST_FIELDS:
        if n not in A:
            A[n] = np.zeros(abi.field_shape(kind, ncol, npatch, ncol), dtype=np.dtype(t))
    return A


def add_soilresis_fields(A):
    """The calc_soilevap_resis components a full state lacks: watfc by the
    field-capacity rule of SoilStateInitTimeConstMod.F90:596-600 (hk = 0.1
    mm/day), frac_sno from frac_sno_eff, and zero-filled dsl / soilbeta."""
    ncol = A["zwt"].shape[0]
    secspday = 86400.0
    A["watfc"] = np.ascontiguousarray(A["watsat"] * (0.1 / (A["hksat"] * secspday)) ** (1.0 / (2.0 * A["bsw"] + 3.0)))
    A["frac_sno"] = np.ascontiguousarray(A["frac_sno_eff"].copy())
    for n in ("dsl", "soilbeta"):
        A[n] = np.zeros(ncol)
    if "soilresis" not in A:
        A["soilresis"] = np.zeros(ncol)
    return A


def add_baregrnd_fields(A, npatch, ngrid):
    """The BareGroundFluxes components a full state lacks: the last step's
    ground roughness for heat / moisture (z0hg = z0qg = z0mg/10, builder's
    choice) and forcing heights at patch level (forc_hgt + roughness, as the
    routine leaves them), soilbeta, and zero-filled outputs."""
    ncol = A["zwt"].shape[0]
    if "watfc" not in A:
        add_soilresis_fields(A)
    A["z0hg"] = np.ascontiguousarray(A["z0mg"] / 10.0)
    A["z0qg"] = A["z0hg"].copy()
    pc = A["patch_column"] - 1
    pg = A["patch_gridcell"] - 1
    A["forc_hgt_u_patch"] = np.ascontiguousarray(A["forc_hgt_u"][pg] + A["z0mg"][pc])
    A["forc_hgt_t_patch"] = np.ascontiguousarray(A["forc_hgt_t"][pg] + A["z0hg"][pc])
    A["forc_hgt_q_patch"] = np.ascontiguousarray(A["forc_hgt_q"][pg] + A["z0qg"][pc])
    A["soilbeta"] = np.ascontiguousarray(np.clip(A["h2osoi_vol"][0] / A["watsat"][0], 0.0, 1.0))
    for (n, kind, t, u) in abi.BAREGRND_FIELDS:
        if n not in A:
            A[n] = np.zeros(abi.field_shape(kind, ncol, npatch, ngrid), dtype=np.dtype(t))
    return A


def add_hydrology_fields(A, rng=None):
    """The water-table / drainage / infiltration components a soil state
    lacks: topographic slope U(0.1, 10) degrees, wtfact U(0.2, 0.6), rain plus
    snowmelt U(0, 1e-4) mm/s, snow capping U(0, 1e-6) mm/s, the top-layer and
    surface-water evaporation, h2osfc_thresh U(5, 30) mm (builder's choices);
    zwt_perched and frost_table start at the water table; zero-filled
    outputs."""
    r = rng if rng is not None else np.random.Generator(np.random.Philox(7))
    ncol = A["zwt"].shape[0]
    A["topo_slope"] = r.uniform(0.1, 10.0, ncol)
    A["wtfact"] = r.uniform(0.2, 0.6, ncol)
    A["qflx_rain_plus_snomelt"] = r.uniform(0.0, 1e-4, ncol)
    A["qflx_snwcp_liq"] = r.uniform(0.0, 1e-6, ncol)
    A["qflx_snow_h2osfc"] = r.uniform(0.0, 1e-6, ncol)
    A["qflx_floodc"] = np.zeros(ncol)
    A["qflx_liqevap_from_top_layer_col"] = r.uniform(0.0, 2e-5, ncol)
    A["qflx_ev_soil_col"] = r.uniform(-1e-6, 2e-5, ncol)
    A["qflx_ev_h2osfc_col"] = r.uniform(0.0, 2e-5, ncol)
    A["frac_h2osfc_nosnow"] = np.clip(A["frac_h2osfc"] * 1.2, 0.0, 1.0) if "frac_h2osfc" in A else np.zeros(ncol)
    A["h2osfc_thresh"] = r.uniform(5.0, 30.0, ncol)
    A["hkdepth"] = 1.0 / r.uniform(1.0, 5.0, ncol)         # 1/fff of the aquifer path (m)
    if "wa" not in A:
        A["wa"] = np.full(ncol, 5000.0)
    A["zwt_perched"] = A["zwt"].copy()
    A["frost_table"] = A["zwt"].copy()
    if "h2osfc" not in A:
        A["h2osfc"] = np.zeros(ncol)
    for (n, kind, t, u) in abi.HYDROLOGY_FIELDS:
        if n not in A:
            A[n] = np.zeros(abi.field_shape(kind, ncol, 1, ncol), dtype=np.dtype(t))
    return A

