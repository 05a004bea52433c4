"""Parameters and seeded synthetic inputs for CanopyFluxes + Photosynthesis.

The reference's parameter file is a git-LFS pointer that is not in the
checkout, so the values below are the CLM5 technical note's
(doc/source/tech_note/Fluxes/CLM50_Tech_Note_Fluxes.rst:1015-1060,
Photosynthesis/CLM50_Tech_Note_Photosynthesis.rst:149-260) and the
reference's module constants; parity is oracle vs kernel on the same values.

Configuration of the canopy workload: z0param_method
= ZengWang2007, use_biomass_heat_storage = .false., satellite phenology (no
CN, no LUNA), no hydraulic stress, Medlyn 2011 stomatal conductance,
light_inhibit = .true., soil resistance sl14 (soilresis given), nlevcan = 1,
itmax_canopy_fluxes = 40 (up to 41 passes).

Workload rules the description leaves to the builder:
* patches: 1-4 per column (uniform), one column per gridcell; PFT 0 is a C3
  broadleaf-like type and PFT 1 a C4 grass, drawn 80:20;
* vegetation: LAI ~ U(0,8), SAI ~ U(0,2), htop ~ U(1,20) m (C3) or U(0.2,1) m
  (C4), displa = 0.67 htop, z0mv = 0.055 htop before the ZengWang blend,
  emv = 1 - exp(-(elai+esai)), fwet ~ U(0,0.3), fdry = (1-fwet) elai/(elai+esai);
* atmosphere: forc_t ~ U(250,315) K, relative humidity ~ U(10,100) %, wind
  ~ U(0.5,20) m/s, reference heights 30 m, CO2 400 ppm, O2 0.209 forc_pbot,
  forc_pbot ~ U(86,101.3) kPa, longwave = eps_a sigma T^4 with eps_a ~ U(0.7,1);
* radiation: absorbed PAR per sunlit leaf area ~ U(0,600) W/m2, shaded 10-50 %
  of it, 10 % of the patches at night (PAR = 0); sunlit fraction ~ U(0.2,0.8);
  vcmaxcint from the two-stream extinction coefficients kn = 0.3, kb = 0.5;
* btran ~ U(0,1); ground: t_grnd = forc_t + U(-5,5), qg = qsat(t_grnd) U(0.5,1),
  30 % of the columns snow covered (frac_sno_eff U(0.2,1), 1-3 snow layers).
"""
import numpy as np

from . import abi

TFRZ = 273.15
SB = 5.67e-8
RAIR = 6.02214e26 * 1.38065e-23 / 28.966
CPAIR = 1.00464e3
HVAP = 2.501e6

DEFAULT_PARAMS = dict(
    lai_dl=0.5, z_dl=0.05, a_coef=0.13, a_exp=0.45, csoilc=0.004, cv=0.01, wind_min=1.0, zetamaxstable=0.5,
    kc25_coef=404.9e-6, ko25_coef=278.4e-3, cp25_yr2000=42.75e-6, kcha=79430.0, koha=36380.0, cpha=37830.0,
    vcmaxha=72000.0, jmaxha=50000.0, tpuha=72000.0, lmrha=46390.0, vcmaxhd=200000.0, jmaxhd=200000.0,
    tpuhd=200000.0, lmrhd=150650.0, lmrse=490.0, vcmaxse_sf=1.0, jmaxse_sf=1.0, tpuse_sf=1.0, jmax25top_sf=1.0,
    fnr=7.16, act25=3.6 * 1000.0 / 60.0, theta_psii=0.7, theta_ip=0.95, tpu25ratio=0.167, kp25ratio=20000.0,
    fnps=0.15, leaf_mr_vcm=0.015, light_inhibit=1)

# (c3psn, slatop, leafcn, flnr, fnitr, dleaf, medlynslope, medlynintercept, theta_cj, mbbopt, smpso, smpsc);
# smpso / smpsc (soil water potential at full stomatal opening / closure, mm)
# are the builder's choice for grasses: the parameter file is not in the
# repository.
DEFAULT_PFT = [
    (1.0, 0.030, 25.0, 0.09, 0.90, 0.04, 4.45, 100.0, 0.9393, 9.0, -74000.0, -275000.0),   # C3
    (0.0, 0.050, 25.0, 0.09, 0.80, 0.04, 1.62, 100.0, 0.80, 4.0, -74000.0, -275000.0),     # C4
]


def make_params(overrides=None):
    d = dict(DEFAULT_PARAMS)
    if overrides:
        d.update(overrides)
    p = abi.CanopyParams()
    for k, v in d.items():
        setattr(p, k, v)
    return p


def make_pftcon(rows=None):
    rows = rows or DEFAULT_PFT
    f = abi.Pftcon()
    f.npft = len(rows)
    names = ["c3psn", "slatop", "leafcn", "flnr", "fnitr", "dleaf", "medlynslope", "medlynintercept", "theta_cj",
             "mbbopt", "smpso", "smpsc"]
    for i, row in enumerate(rows):
        for n, v in zip(names, row):
            getattr(f, n)[i] = v
    return f


def qsat(T, p):
    """QSat (QSatMod.F90:61-127) in numpy, for input preparation only."""
    a = [6.11213476, 0.444007856, 0.143064234e-01, 0.264461437e-03, 0.305903558e-05, 0.196237241e-07,
         0.892344772e-10, -0.373208410e-12, 0.209339997e-15]
    c = [6.11123516, 0.503109514, 0.188369801e-01, 0.420547422e-03, 0.614396778e-05, 0.602780717e-07,
         0.387940929e-09, 0.149436277e-11, 0.262655803e-14]
    b = [0.444017302, 0.286064092e-01, 0.794683137e-03, 0.121211669e-04, 0.103354611e-06, 0.404125005e-09,
         -0.788037859e-12, -0.114596802e-13, 0.381294516e-16]
    d = [0.503277922, 0.377289173e-01, 0.126801703e-02, 0.249468427e-04, 0.313703411e-06, 0.257180651e-08,
         0.133268878e-10, 0.394116744e-13, 0.498070196e-16]
    td = np.clip(T - TFRZ, -75.0, 100.0)

    def horner(co):
        r = np.zeros_like(td) + co[8]
        for k in range(7, -1, -1):
            r = co[k] + td * r
        return r
    es = np.where(td >= 0, horner(a), horner(c)) * 100.0
    esdT = np.where(td >= 0, horner(b), horner(d)) * 100.0
    vp = 1.0 / (p - 0.378 * es)
    qs = es * 0.622 * vp
    return qs, es, esdT * 0.622 * vp * vp * p


def canopy_patches(npatch, seed=0, npatch_max=4, night_frac=0.1, rng=None):
    """Allocate and fill every canopy manifest field for about `npatch`
    patches (1..npatch_max per column).  Returns (arrays, npatch, ncol, ngrid)."""
    r = rng if rng is not None else np.random.Generator(np.random.Philox(seed))
    per = r.integers(1, npatch_max + 1, npatch).astype(np.int32)
    ncut = int(np.searchsorted(np.cumsum(per), npatch)) + 1      # first prefix reaching npatch
    per = per[:ncut]
    per[-1] -= int(per.sum()) - npatch
    ncol = len(per)
    ngrid = ncol
    A = {}
    for (n, kind, dt, use) in abi.CANOPY_FIELDS:
        A[n] = np.zeros(abi.field_shape(kind, ncol, npatch, ngrid), dtype=np.dtype(dt))
    pcol = np.repeat(np.arange(ncol), per)
    A["patch_column"][:] = pcol + 1
    A["patch_gridcell"][:] = pcol + 1
    c3 = r.uniform(0, 1, npatch) < 0.8
    A["itype"][:] = np.where(c3, 0, 1)

    # gridcell / column atmosphere
    forc_t = r.uniform(250.0, 315.0, ncol)
    rh = r.uniform(0.10, 1.00, ncol)
    wind = r.uniform(0.5, 20.0, ncol)
    pbot = r.uniform(86000.0, 101325.0, ncol)
    qs, es, _ = qsat(forc_t, pbot)
    forc_q = rh * qs
    A["forc_u"][:] = wind
    A["forc_v"][:] = 0.0
    for k in ("forc_hgt_u", "forc_hgt_t", "forc_hgt_q"):
        A[k][:] = 30.0
    A["forc_pco2"][:] = 400.e-6 * pbot
    A["forc_po2"][:] = 0.209 * pbot
    A["dayl"][:] = r.uniform(28800.0, 57600.0, ngrid)
    A["max_dayl"][:] = 57600.0
    A["forc_pbot"][:] = pbot
    A["forc_q"][:] = forc_q
    forc_th = forc_t * (100000.0 / pbot) ** (RAIR / CPAIR)
    A["forc_th"][:] = forc_th
    e = forc_q * pbot / (0.622 + 0.378 * forc_q)
    A["forc_rho"][:] = (pbot - 0.378 * e) / (RAIR * forc_t)
    A["forc_lwrad"][:] = r.uniform(0.7, 1.0, ncol) * SB * forc_t ** 4
    A["thv"][:] = forc_th * (1.0 + 0.61 * forc_q)

    # ground
    t_grnd = forc_t + r.uniform(-5.0, 5.0, ncol)
    A["t_grnd"][:] = t_grnd
    qg_s, _, qgdT = qsat(t_grnd, pbot)
    wet = r.uniform(0.5, 1.0, ncol)
    A["qg"][:] = qg_s * wet
    A["qg_snow"][:] = qg_s
    A["qg_soil"][:] = qg_s * wet
    A["qg_h2osfc"][:] = qg_s
    A["dqgdT"][:] = qgdT * wet
    A["emg"][:] = 0.96
    A["htvp"][:] = HVAP
    A["z0mg"][:] = 0.01
    snowy = r.uniform(0, 1, ncol) < 0.3
    snl = np.where(snowy, -r.integers(1, 4, ncol), 0).astype(np.int32)
    A["snl"][:] = snl
    A["frac_sno_eff"][:] = np.where(snowy, r.uniform(0.2, 1.0, ncol), 0.0)
    A["snow_depth"][:] = np.where(snowy, r.uniform(0.01, 0.3, ncol), 0.0)
    A["frac_h2osfc"][:] = 0.0
    A["soilresis"][:] = r.uniform(50.0, 5000.0, ncol)
    A["t_h2osfc"][:] = t_grnd
    LS = -abi.NLEVSNO + 1
    tsoi = A["t_soisno"]
    tsoi[1 - LS] = t_grnd + r.uniform(-1.0, 1.0, ncol)
    for j in range(-2, 1):
        tsoi[j - LS] = np.where(j >= snl + 1, np.minimum(t_grnd, TFRZ) + r.uniform(-2.0, 0.0, ncol), 0.0)

    # patches
    fp = lambda a: a[pcol]
    lai = r.uniform(0.0, 8.0, npatch)
    lai = np.maximum(lai, 1e-3)
    sai = r.uniform(0.0, 2.0, npatch)
    A["elai"][:] = lai
    A["esai"][:] = sai
    htop = np.where(c3, r.uniform(1.0, 20.0, npatch), r.uniform(0.2, 1.0, npatch))
    A["htop"][:] = htop
    A["displa"][:] = 0.67 * htop
    A["z0mv"][:] = 0.055 * htop
    A["emv"][:] = 1.0 - np.exp(-(lai + sai))
    fwet = r.uniform(0.0, 0.3, npatch)
    A["fwet"][:] = fwet
    A["fdry"][:] = (1.0 - fwet) * lai / (lai + sai)
    fsun = r.uniform(0.2, 0.8, npatch)
    A["laisun"][:] = fsun * lai
    A["laisha"][:] = (1.0 - fsun) * lai
    A["btran"][:] = r.uniform(0.0, 1.0, npatch)
    par = r.uniform(0.0, 600.0, npatch)
    night = r.uniform(0, 1, npatch) < night_frac
    par = np.where(night, 0.0, par)
    A["parsun_z"][:] = par
    A["parsha_z"][:] = par * r.uniform(0.1, 0.5, npatch)
    A["sabv"][:] = 2.0 * (A["parsun_z"] * A["laisun"] + A["parsha_z"] * A["laisha"]) / np.maximum(lai, 1.0)
    kn, kb = 0.3, 0.5
    vsun = (1.0 - np.exp(-(kn + kb) * lai)) / (kn + kb)
    vsha = (1.0 - np.exp(-kn * lai)) / kn - vsun
    A["vcmaxcintsun"][:] = vsun / (fsun * lai)
    A["vcmaxcintsha"][:] = vsha / ((1.0 - fsun) * lai)
    A["thm"][:] = fp(forc_t) + 0.0098 * 30.0
    A["t_a10"][:] = fp(forc_t) + r.uniform(-3.0, 3.0, npatch)
    A["t_veg"][:] = fp(forc_t) + r.uniform(-2.0, 2.0, npatch)
    A["liqcan"][:] = r.uniform(0.0, 0.5, npatch)
    A["snocan"][:] = np.where(A["t_veg"] < TFRZ, r.uniform(0.0, 0.5, npatch), 0.0)
    A["frac_veg_nosno"][:] = 1
    A["cgrnds"][:] = 0.0
    A["cgrndl"][:] = 0.0
    return A, npatch, ncol, ngrid
