"""Seeded synthetic column inputs for the soil path (no dataset is involved).

All draws come from one numpy Philox generator per seed, so the oracle and the
GPU see identical inputs.  The rules that the workload description leaves to
the builder are stated here and nowhere else:

* layer structure 20SL_8.5m (src/main/initVerticalMod.F90:291-318):
  dz_j = 0.02 j (j<=4), dz_4 + 0.04 (j-4) (j<=13), dz_13 + 0.10 (j-13) (j<=20),
  dz_20 + ((j-20)*25)^1.5/100 for the five bedrock layers;
* soil properties: one sand / clay / organic-matter triple per column used for
  all levels, fed through the Cosby (1984) table-5 pedotransfer with organic
  mixing of src/biogeophys/SoilStateInitTimeConstMod.F90:541-602; default
  parameter values (tkd_sand 8.80, tkd_clay 2.92, tkm_om 0.25, tkd_om 0.05,
  csol_sand 2.128, csol_clay 2.385, csol_om 2.5, pd 2700, organic_max 130,
  every *_sf = 1) come from the CLM5 technical note because the parameter
  file is not available;
* soil water: h2osoi_vol ~ U(0.05, watsat) on levels 1..nlevsoi, zero below;
  a layer colder than tfrz holds a frozen fraction min(0.9, (tfrz-T)/10) of
  that volume as ice;
* soil temperature: U(265,300) K plus a per-column gradient U(-0.02,0.02) K/cm
  applied down to the bottom of the soil column (8.6 m) and held constant in
  the bedrock below;
* snow (when enabled): layer thickness U(0.01,0.5) m, bulk density
  U(50,400) kg/m3, liquid fraction U(0,0.1) of the snow water, temperature
  U(230,273.15) K, frac_sno_eff = 1 on snow columns;
* forcing: qflx_infl U(0,2e-4) mm/s; a transpiration sink U(0,1e-4) mm/s split
  over the 20 soil layers by the fixed profile dz_j exp(-3 z_j) (normalised);
  zwt U(0.5,8) m; the ground heat flux G ~ U(-50,150) W/m2 enters as one patch
  per column with wtcol = 1, emg = 0, sabg = sabg_soil = sabg_snow = G, all of it
  absorbed in the top layer, the turbulent fluxes at zero and cgrnd = 5 W/m2/K
  (forcing="full": sabg = sabg_soil = sabg_snow drawn per patch and split over
  the exposed layers, every other patch flux drawn independently);
  eflx_bot = 0, h2osfc = frac_h2osfc = 0.
"""
import numpy as np

from .abi import NLEVSNO, NLEVSOI, NLEVGRND, SOILWATER_FIELDS, SOILWATER_EXTRA, SOILTEMP_FIELDS, field_shape

TFRZ = 273.15
DENH2O = 1.000e3
DENICE = 0.917e3
HVAP = 2.501e6
SECSPDAY = 86400.0

ORGANIC_MAX = 130.0
PEDO = dict(tkd_sand=8.80, tkd_clay=2.92, tkm_om=0.25, tkd_om=0.05, csol_sand=2.128,
            csol_clay=2.385, csol_om=2.5, pd=2700.0, zsapric=0.5, pcalpha=0.5, pcbeta=0.139)

ALL_FIELDS = {}
for _f in SOILWATER_FIELDS + SOILWATER_EXTRA + SOILTEMP_FIELDS:
    ALL_FIELDS[_f[0]] = _f


def layer_structure_20sl():
    """dzsoi, zsoi, zisoi(0:nlevgrnd) of 20SL_8.5m (initVerticalMod.F90:291-318)."""
    dz = np.zeros(NLEVGRND + 1)
    for j in range(1, 5):
        dz[j] = j * 0.02
    for j in range(5, 14):
        dz[j] = dz[4] + (j - 4) * 0.04
    for j in range(14, NLEVSOI + 1):
        dz[j] = dz[13] + (j - 13) * 0.10
    for j in range(NLEVSOI + 1, NLEVGRND + 1):
        dz[j] = dz[NLEVSOI] + (((j - NLEVSOI) * 25.0) ** 1.5) / 100.0
    zi = np.zeros(NLEVGRND + 1)
    for j in range(1, NLEVGRND + 1):
        s = 0.0
        for k in range(1, j + 1):      # Fortran sum(dzsoi(1:j)), left to right
            s = s + dz[k]
        zi[j] = s
    z = np.zeros(NLEVGRND + 1)
    for j in range(1, NLEVGRND + 1):
        z[j] = 0.5 * (zi[j - 1] + zi[j])
    return dz[1:], z[1:], zi


def pedotransfer(sand, clay, om, zsoi):
    """Soil hydraulic and thermal properties per level
    (SoilStateInitTimeConstMod.F90:446-602, FuncPedotransferMod.F90:83-103).
    sand, clay in %, om in kg/m3 (arrays over columns); returns dict of
    (nlevgrnd, ncol) arrays."""
    P = PEDO
    ncol = sand.shape[0]
    out = {k: np.empty((NLEVGRND, ncol)) for k in ("watsat", "bsw", "sucsat", "hksat", "tkmg",
                                                    "tksatu", "tkdry", "csol")}
    for lev in range(1, NLEVGRND + 1):
        om_frac = np.minimum(1.0 * om / ORGANIC_MAX, 1.0) if lev <= NLEVSOI else np.zeros(ncol)
        watsat = 0.489 - 0.00126 * sand
        xksat = 0.0070556 * (10.0 ** (-0.884 + 0.0153 * sand))
        sucsat = 10.0 * (10.0 ** (1.88 - 0.0131 * sand))
        zs = zsoi[lev - 1]
        om_watsat = max(0.93 - 0.1 * (zs / P["zsapric"]), 0.83)
        om_b = min(2.7 + 9.3 * (zs / P["zsapric"]), 12.0)
        om_sucsat = min(10.3 - 0.2 * (zs / P["zsapric"]), 10.1)
        om_hksat = np.maximum(0.28 - 0.2799 * (zs / P["zsapric"]), xksat)
        bd = (1.0 - watsat) * P["pd"]
        watsat = np.minimum(1.0 * ((1.0 - om_frac) * watsat + om_watsat * om_frac), 0.93)
        tkm = (1.0 - om_frac) * (P["tkd_sand"] * sand + P["tkd_clay"] * clay) / (sand + clay) + P["tkm_om"] * om_frac
        bsw = 1.0 * ((1.0 - om_frac) * (2.91 + 0.159 * clay) + om_frac * om_b)
        sucsat = 1.0 * ((1.0 - om_frac) * sucsat + om_sucsat * om_frac)
        perc_norm = (1.0 - P["pcalpha"]) ** (-P["pcbeta"])
        perc_frac = np.where(om_frac > P["pcalpha"],
                             perc_norm * np.maximum(om_frac - P["pcalpha"], 0.0) ** P["pcbeta"], 0.0)
        uncon_frac = (1.0 - om_frac) + (1.0 - perc_frac) * om_frac
        with np.errstate(divide="ignore", invalid="ignore"):
            uncon_hksat = np.where(om_frac < 1.0,
                                   uncon_frac / ((1.0 - om_frac) / xksat + ((1.0 - perc_frac) * om_frac) / om_hksat),
                                   0.0)
        hksat = 1.0 * (uncon_frac * uncon_hksat + (perc_frac * om_frac) * om_hksat)
        tkmg = tkm ** (1.0 - watsat)
        tksatu = tkmg * 0.57 ** watsat
        tkdry = ((0.135 * bd + 64.7) / (P["pd"] - 0.947 * bd)) * (1.0 - om_frac) + P["tkd_om"] * om_frac
        csol = ((1.0 - om_frac) * (P["csol_sand"] * sand + P["csol_clay"] * clay) / (sand + clay) +
                P["csol_om"] * om_frac) * 1.e6
        for k, v in (("watsat", watsat), ("bsw", bsw), ("sucsat", sucsat), ("hksat", hksat),
                     ("tkmg", tkmg), ("tksatu", tksatu), ("tkdry", tkdry), ("csol", csol)):
            out[k][lev - 1] = v
    return out


def _rng(seed):
    return np.random.Generator(np.random.Philox(seed))


def soil_columns(ncol, seed=0, snow=False, nbedrock=(20, 20), zwt=(0.5, 8.0),
                 forcing="ground_flux", npatch_max=1, h2osfc=False, rng=None):
    """Allocate and fill every manifest field for `ncol` columns.

    snow=False gives snl = 0 everywhere; snow=True draws snl ~ U{0..-12}.
    nbedrock=(lo, hi) draws U{lo..hi}.  forcing="ground_flux" is the workload
    rule in the module docstring; forcing="full" (tests) draws every patch flux,
    emissivity and longwave independently and 1..npatch_max patches per column;
    h2osfc=True (tests) adds standing surface water.
    Returns (arrays, npatch)."""
    r = rng if rng is not None else _rng(seed)
    dzs, zs, zis = layer_structure_20sl()
    LS = -NLEVSNO + 1

    if forcing == "full":
        npc = r.integers(1, npatch_max + 1, size=ncol).astype(np.int32)
    else:
        npc = np.ones(ncol, dtype=np.int32)
    npatch = int(npc.sum())
    A = {}
    for name, (n, kind, dt, use) in ALL_FIELDS.items():
        A[name] = np.zeros(field_shape(kind, ncol, npatch), dtype=np.dtype(dt))

    # ---- geometry
    snl = (-r.integers(0, NLEVSNO + 1, size=ncol)).astype(np.int32) if snow else np.zeros(ncol, np.int32)
    A["snl"][:] = snl
    A["nbedrock"][:] = r.integers(nbedrock[0], nbedrock[1] + 1, size=ncol)
    for j in range(1, NLEVGRND + 1):
        A["dz"][j - LS] = dzs[j - 1]
        A["z"][j - LS] = zs[j - 1]
        A["zi"][j + NLEVSNO] = zis[j]
    A["zi"][0 + NLEVSNO] = 0.0
    sdz = r.uniform(0.01, 0.5, size=(NLEVSNO, ncol))           # snow layer j = -11..0 at row j+11
    sden = r.uniform(50.0, 400.0, size=(NLEVSNO, ncol))
    sliqf = r.uniform(0.0, 0.1, size=(NLEVSNO, ncol))
    stemp = r.uniform(230.0, TFRZ, size=(NLEVSNO, ncol))
    for j in range(0, LS - 1, -1):
        act = j >= snl + 1
        row = j - LS
        dzj = np.where(act, sdz[row], 0.0)
        A["dz"][row] = dzj
        zij = A["zi"][j + NLEVSNO]
        A["zi"][j - 1 + NLEVSNO] = np.where(act, zij - dzj, 0.0)
        A["z"][row] = np.where(act, zij - 0.5 * dzj, 0.0)
        tot = sden[row] * dzj
        A["h2osoi_liq"][row] = np.where(act, sliqf[row] * tot, 0.0)
        A["h2osoi_ice"][row] = np.where(act, (1.0 - sliqf[row]) * tot, 0.0)
        A["t_soisno"][row] = np.where(act, stemp[row], 0.0)
    has_snow = snl < 0
    A["frac_sno_eff"][:] = np.where(has_snow, 1.0, 0.0)
    A["snow_depth"][:] = -A["zi"][snl + NLEVSNO, np.arange(ncol)]
    A["int_snow"][:] = (A["h2osoi_liq"][:NLEVSNO] + A["h2osoi_ice"][:NLEVSNO]).sum(axis=0)

    # ---- soil properties
    while True:
        sand = r.uniform(5.0, 85.0, size=ncol)
        clay = r.uniform(5.0, 85.0, size=ncol)
        bad = sand + clay > 95.0
        if not bad.any():
            break
        # rejection sampling, column by column, keeps the draw reproducible
        for i in np.nonzero(bad)[0]:
            while sand[i] + clay[i] > 95.0:
                sand[i] = r.uniform(5.0, 85.0)
                clay[i] = r.uniform(5.0, 85.0)
        break
    om = r.uniform(0.0, 130.0, size=ncol)
    props = pedotransfer(sand, clay, om, zs)
    for k in ("watsat", "bsw", "sucsat", "hksat", "tkmg", "tkdry", "csol"):
        A[k][:] = props[k]
    A["smpmin"][:] = -1.e8

    # ---- soil state
    t0 = r.uniform(265.0, 300.0, size=ncol)
    grad = r.uniform(-0.02, 0.02, size=ncol)
    vol = r.uniform(0.0, 1.0, size=(NLEVSOI, ncol))
    for j in range(1, NLEVGRND + 1):
        row = j - LS
        depth = min(zs[j - 1], zis[NLEVSOI])
        T = t0 + grad * 100.0 * depth
        A["t_soisno"][row] = T
        if j <= NLEVSOI:
            ws = A["watsat"][j - 1]
            v = 0.05 + vol[j - 1] * (ws - 0.05)
            fice = np.clip((TFRZ - T) / 10.0, 0.0, 0.9)
            A["h2osoi_liq"][row] = (1.0 - fice) * v * dzs[j - 1] * DENH2O
            A["h2osoi_ice"][row] = fice * v * dzs[j - 1] * DENICE
            A["h2osoi_vol"][j - 1] = v
    A["t_h2osfc"][:] = A["t_soisno"][1 - LS]
    top = snl + 1
    A["t_grnd"][:] = A["t_soisno"][top - LS, np.arange(ncol)]

    # ---- hydrology forcing
    A["qflx_infl"][:] = r.uniform(0.0, 2e-4, size=ncol)
    prof = np.array([dzs[j] * np.exp(-3.0 * zs[j]) for j in range(NLEVSOI)])
    prof = prof / prof.sum()
    tran = r.uniform(0.0, 1e-4, size=ncol)
    A["qflx_rootsoi"][:] = prof[:, None] * tran[None, :]
    A["zwt"][:] = r.uniform(zwt[0], zwt[1], size=ncol)

    # ---- energy forcing
    pstart = np.concatenate([[0], np.cumsum(npc)[:-1]]).astype(np.int32)
    A["col_patchi"][:] = pstart + 1          # 1-based global patch index, begp = 1
    A["col_npatches"][:] = npc
    A["htvp"][:] = HVAP
    A["eflx_bot"][:] = 0.0
    pcol = np.repeat(np.arange(ncol), npc)
    if forcing == "ground_flux":
        G = r.uniform(-50.0, 150.0, size=ncol)
        A["emg"][:] = 0.0
        A["forc_lwrad"][:] = 300.0
        A["wtcol"][:] = 1.0
        for k in ("sabg", "sabg_soil", "sabg_snow"):
            A[k][:] = G
        A["sabg_lyr"][top - LS, np.arange(ncol)] = G
        A["cgrnd"][:] = 5.0
    else:
        w = r.uniform(0.1, 1.0, size=npatch)
        wsum = np.bincount(pcol, weights=w, minlength=ncol)
        A["wtcol"][:] = w / wsum[pcol]
        A["frac_veg_nosno"][:] = r.integers(0, 2, size=npatch)
        A["emg"][:] = r.uniform(0.9, 0.99, size=ncol)
        A["forc_lwrad"][:] = r.uniform(150.0, 450.0, size=ncol)
        A["sabg"][:] = r.uniform(0.0, 400.0, size=npatch)
        A["sabg_soil"][:] = A["sabg"]
        A["sabg_snow"][:] = A["sabg"]
        frac = r.uniform(0.0, 1.0, size=(NLEVSNO + 1, npatch))
        ptop = top[pcol]
        for j in range(LS, 2):
            A["sabg_lyr"][j - LS] = np.where(j >= ptop, frac[j - LS], 0.0)
        tot = A["sabg_lyr"].sum(axis=0)
        A["sabg_lyr"][:] = A["sabg_lyr"] / tot[None, :] * A["sabg"][None, :]
        A["dlrad"][:] = r.uniform(0.0, 100.0, size=npatch)
        for k in ("eflx_sh_grnd", "eflx_sh_snow", "eflx_sh_soil", "eflx_sh_h2osfc"):
            A[k][:] = r.uniform(-50.0, 150.0, size=npatch)
        for k in ("qflx_evap_soi", "qflx_ev_snow", "qflx_ev_soil", "qflx_ev_h2osfc"):
            A[k][:] = r.uniform(-1e-5, 5e-5, size=npatch)
        A["cgrnd"][:] = r.uniform(1.0, 30.0, size=npatch)
        A["eflx_bot"][:] = r.uniform(-0.1, 0.1, size=ncol)
    if h2osfc:
        A["h2osfc"][:] = r.uniform(0.0, 50.0, size=ncol)
        A["frac_h2osfc"][:] = np.where(has_snow, r.uniform(0.0, 0.3, size=ncol), r.uniform(0.0, 0.6, size=ncol))
        A["frac_h2osfc"][:] = np.minimum(A["frac_h2osfc"], 1.0 - A["frac_sno_eff"])
        A["frac_sno_eff"][:] = np.where(has_snow, 1.0 - A["frac_h2osfc"], 0.0)
        A["t_h2osfc"][:] = r.uniform(268.0, 285.0, size=ncol)
    A["wa"][:] = 5000.0      # aquifer water at aquifer_water_baseline (clm_varcon.F90:124)
    set_soil_water_fractions(A)
    return A, npatch


def set_soil_water_fractions(A):
    """icefrac and eff_porosity on levels 1..nlevsoi as SetSoilWaterFractions
    computes them before SoilWater (SoilHydrologyMod.F90:236-249, no excess
    ice: dz_ext = dz)."""
    LS = -NLEVSNO + 1
    for j in range(1, NLEVSOI + 1):
        row = j - LS
        ws = A["watsat"][j - 1]
        vol_ice = np.minimum(ws, (A["h2osoi_ice"][row] + 0.0) / ((A["dz"][row] + 0.0 / DENICE) * DENICE))
        A["eff_porosity"][j - 1] = np.maximum(0.01, ws - vol_ice)
        A["icefrac"][j - 1] = np.minimum(1.0, vol_ice / ws)


def refresh_h2osoi_vol(A):
    """h2osoi_vol = liq/(dz denh2o) + ice/(dz denice) on levels 1..nlevsoi, the
    update the driver makes between steps (HydrologyNoDrainageMod.F90:580,590)."""
    LS = -NLEVSNO + 1
    for j in range(1, NLEVSOI + 1):
        row = j - LS
        dz = A["dz"][row]
        A["h2osoi_vol"][j - 1] = A["h2osoi_liq"][row] / (dz * DENH2O) + A["h2osoi_ice"][row] / (dz * DENICE)
