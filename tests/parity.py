"""Helpers for comparing the CUDA path with the oracle."""
import numpy as np

# Cancellation diagnostics: the inter-layer Darcy fluxes (qin, qout =
# -hk*((smp_j - smp_{j-1}) - (zq_j - zq_{j-1}))/dz, SoilWaterMovementMod.F90:801-894)
# and the interface heat fluxes (eflx_fgr = -cnfac*fn - (1-cnfac)*fn1 with
# fn = tk*(T_{j+1}-T_j)/dz, SoilTemperatureMod.F90:438-504) and the latent heat
# of phase change (xmf = hfus*(wice0 - h2osoi_ice)/dtime summed over layers,
# SoilTemperatureMod.F90:1492-1502) are differences of nearly equal operands, so their elementwise relative error is set by the
# operands, not by the result (in ZD09 the equilibrium profile zq itself comes
# from the difference of two close pow() values, :686-705).  For these the
# acceptance test is the reference's own conditioning: an element passes when
# |gpu - oracle| is within 1e-9*|oracle| plus the spread of the oracle itself
# when every libm result (pow, log10) it uses is perturbed independently by up
# to NOISE_ULPS ulp (NOISE_RUNS realisations).  CUDA's double pow is within
# 2 ulp of the correctly rounded result and glibc's within 1 ulp, so the two
# implementations differ by at most 3 ulp per call.
CANCELLATION = ("qin", "qout", "eflx_fgr", "xmf")
NOISE_ULPS = 4
NOISE_RUNS = 4


def max_rel_err(a, b, floor_frac=1e-12):
    """Elementwise relative error |a-b| / (|b| + floor), floor = floor_frac *
    max|b| over the field (so that exact zeros and round-off-sized values of a
    field whose scale is set by its large entries do not divide by ~0)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.size == 0:
        return 0.0
    scale = np.nanmax(np.abs(b)) if np.isfinite(b).any() else 0.0
    floor = floor_frac * scale + 1e-300
    d = np.abs(a - b)
    both_nan = np.isnan(a) & np.isnan(b)
    d = np.where(both_nan, 0.0, d)
    return float(np.nanmax(d / (np.abs(b) + floor))) if d.size else 0.0


def perturb_inputs(A, ulps, seed, skip=()):
    """Copy of A with every float64 array scaled elementwise by (1 + k eps),
    k uniform in [-ulps, ulps]: a stand-in for the rounding differences of
    the intermediate operations (FMA contraction on the device)."""
    import copy
    r = np.random.Generator(np.random.Philox(10_000 + seed))
    B = copy.deepcopy(A)
    eps = np.finfo(np.float64).eps
    for k, v in B.items():
        if v.dtype == np.float64 and k not in skip:
            B[k] = v * (1.0 + eps * r.integers(-ulps, ulps + 1, size=v.shape))
    return B


def noise_spread(run, A, R, fields=CANCELLATION, input_ulps=0):
    """Per-element spread of the oracle's outputs `fields` under libm noise
    (and, if input_ulps > 0, an independent +-input_ulps perturbation of every
    floating-point input).  run(B) runs the oracle in place on a copy B of the
    inputs A; R is the noise-free result."""
    import copy
    from oracle import oracle as orc
    L = orc.lib()
    out = {k: np.zeros_like(R[k]) for k in fields}
    try:
        for seed in range(1, NOISE_RUNS + 1):
            L.oracle_set_libm_noise(NOISE_ULPS, seed)
            B = perturb_inputs(A, input_ulps, seed) if input_ulps else copy.deepcopy(A)
            run(B)
            for k in fields:
                out[k] = np.maximum(out[k], np.abs(B[k] - R[k]))
    finally:
        L.oracle_set_libm_noise(0, 0)
    return out


def fgr_rounding_bound(R, ulps=8):
    """Absolute error bound of eflx_fgr(j) (j = 1..nlevgrnd) that comes from the
    rounding of the new temperatures alone: (1-cnfac) * tk_j * ulps * eps *
    (|T_j| + |T_{j+1}|) / (z_{j+1} - z_j), with tk_j the interface conductivity
    of SoilTemperatureMod.F90:822-828 evaluated from the oracle's thk."""
    from ctsm_gb300.abi import NLEVSNO, NLEVGRND
    eps = np.finfo(np.float64).eps
    LS = -NLEVSNO + 1
    out = np.zeros_like(R["eflx_fgr"])
    for j in range(1, NLEVGRND):
        r, rp = j - LS, j + 1 - LS
        t1, t2 = R["thk"][r], R["thk"][rp]
        z1, z2, zi = R["z"][r], R["z"][rp], R["zi"][j + NLEVSNO]
        tk = t1 * t2 * (z2 - z1) / (t1 * (z2 - zi) + t2 * (zi - z1))
        out[j - 1] = 0.5 * np.abs(tk) * ulps * eps * (np.abs(R["t_soisno"][r]) + np.abs(R["t_soisno"][rp])) / (z2 - z1)
    return out


def conditioned_excess(g, r0, spread):
    """max over elements of (|g-r0| - spread) / (1e-9 |r0| + tiny); <= 1 passes."""
    d = np.abs(np.asarray(g) - np.asarray(r0)) - spread
    scale = 1e-9 * np.abs(r0) + 1e-300 + 1e-21 * np.nanmax(np.abs(r0))
    return float(np.nanmax(np.maximum(d, 0.0) / scale)) * 1e-9


def compare(gpu, ref, fields, tol=1e-9, spread=None):
    """Return {field: max error} and the list of fields above tol.  Integer
    fields count mismatching elements; cancellation diagnostics use the
    conditioned test when `spread` (field -> oracle spread array) is given."""
    errs = {}
    for k in fields:
        g, r = gpu[k], ref[k]
        if g.dtype.kind == "i":
            errs[k] = float(np.count_nonzero(g != r))
        elif spread is not None and k in spread:
            errs[k] = conditioned_excess(g, r, spread[k])
        else:
            errs[k] = max_rel_err(g, r)
    bad = [k for k, v in errs.items() if v > tol]
    return errs, bad


def evap_veg_rounding_bound(R, ulps=8):
    """Absolute error of qflx_evap_veg = rpp * efpot that the rounding of
    efpot's operands allows: efpot = forc_rho (elai + esai) / rb
    (wtgaq (qsatl + qsatldT dt_veg) - wtgq0 qg - wtaq0 forc_q)
    (CanopyFluxesMod.F90:1335-1339) is a difference of humidities the size of
    the canopy-air humidity qaf, so near saturation its sign is set by
    rounding: ulps * eps * forc_rho (elai + esai) / rb1 * (|qaf| + |forc_q|),
    per patch, from the oracle's state R."""
    eps = np.finfo(np.float64).eps
    c = R["patch_column"] - 1
    return ulps * eps * R["forc_rho"][c] * (R["elai"] + R["esai"]) / R["rb1"] * (np.abs(R["qaf"]) +
                                                                                  np.abs(R["forc_q"][c]))
