"""Soil-property preparation (ctsm_gb300.inputs.pedotransfer, the host form
of SoilStateInitTimeConstMod.F90:446-602 with the default Cosby 1984 table 5
pedotransfer function, FuncPedotransferMod.F90:83-103) against an independent
scalar restatement that evaluates the reference's own expressions as pinned
in tests/golden/pedotransfer.json (read from the reference's source text by
tests/golden/make_golden.py).  The parameter-file values (tkd_sand,
csol_sand, pd, ...) are absent from the reference checkout and are the
builder's choices in inputs.PEDO; the structure and every coefficient in the
source text are the reference's."""
import json
import os

import numpy as np

from ctsm_gb300 import inputs

HERE = os.path.dirname(os.path.abspath(__file__))
G = json.load(open(os.path.join(HERE, "golden", "pedotransfer.json")))


def _py(expr):
    """A pinned Fortran expression as Python over scalars."""
    for a, b in (("soilstate_inst%bd_col(c,lev)", "bd"), ("soilstate_inst%tkmg_col(c,lev)", "tkmg"),
                 ("soilstate_inst%watsat_col(c,lev)", "watsat"), ("params_inst%pd", "pd"),
                 ("params_inst%tkd_om", "tkd_om"), ("params_inst%bsw_sf", "1.0"), ("params_inst%watsat_sf", "1.0"),
                 ("zsoi(lev)", "zs"), ("_r8", "")):
        expr = expr.replace(a, b)
    return compile(expr, "<pinned>", "eval")


E = {k: _py(v) for k, v in list(G["table5"].items()) + list(G["organic"].items())}
for k in ("tkdry", "tksatu", "bsw", "watsat"):
    E["final_" + k] = _py(G[k])
C = {k: eval(_py(v)) for k, v in G["constants"].items()}


def restated(sand, clay, om, zs, lev):
    """One level of one column, statement by statement."""
    P = inputs.PEDO
    om_frac = min(1.0 * om / inputs.ORGANIC_MAX, 1.0) if lev <= inputs.NLEVSOI else 0.0
    env = dict(sand=sand, clay=clay, zs=zs, zsapric=C["zsapric"], om_frac=om_frac, pd=P["pd"], tkd_om=P["tkd_om"],
               max=max, min=min)
    watsat = eval(E["watsat"], env)
    bsw = eval(E["bsw"], env)
    sucsat = eval(E["sucsat"], env)
    xksat = eval(E["xksat"], env)
    env["xksat"] = xksat
    om_watsat, om_b = eval(E["om_watsat"], env), eval(E["om_b"], env)
    om_sucsat, om_hksat = eval(E["om_sucsat"], env), eval(E["om_hksat"], env)
    bd = (1.0 - watsat) * P["pd"]
    env.update(bd=bd, watsat=watsat, om_watsat=om_watsat, om_b=om_b)
    watsat = eval(E["final_watsat"], env)
    tkm = (1.0 - om_frac) * (P["tkd_sand"] * sand + P["tkd_clay"] * clay) / (sand + clay) + P["tkm_om"] * om_frac
    bsw = eval(E["final_bsw"], env)
    sucsat = 1.0 * ((1.0 - om_frac) * sucsat + om_sucsat * om_frac)
    if om_frac > C["pcalpha"]:
        perc_frac = (1.0 - C["pcalpha"]) ** (-C["pcbeta"]) * (om_frac - C["pcalpha"]) ** C["pcbeta"]
    else:
        perc_frac = 0.0
    uncon_frac = (1.0 - om_frac) + (1.0 - perc_frac) * om_frac
    if om_frac < 1.0:
        uncon_hksat = uncon_frac / ((1.0 - om_frac) / xksat + ((1.0 - perc_frac) * om_frac) / om_hksat)
    else:
        uncon_hksat = 0.0
    hksat = 1.0 * (uncon_frac * uncon_hksat + (perc_frac * om_frac) * om_hksat)
    tkmg = tkm ** (1.0 - watsat)
    env.update(tkmg=tkmg, watsat=watsat, bd=bd)
    tksatu = eval(E["final_tksatu"], env)
    tkdry = eval(E["final_tkdry"], env)
    csol = ((1.0 - om_frac) * (P["csol_sand"] * sand + P["csol_clay"] * clay) / (sand + clay) +
            P["csol_om"] * om_frac) * 1.e6
    return dict(watsat=watsat, bsw=bsw, sucsat=sucsat, hksat=hksat, tkmg=tkmg, tksatu=tksatu, tkdry=tkdry, csol=csol)


def test_pedotransfer_matches_pinned_restatement():
    r = np.random.Generator(np.random.Philox(17))
    n = 200
    sand = r.uniform(5.0, 85.0, n)
    clay = np.minimum(r.uniform(5.0, 85.0, n), 95.0 - sand)
    om = r.uniform(0.0, 130.0, n)
    om[:20] = 0.0                              # mineral soil: the table-5 expressions alone
    om[20:30] = 130.0                          # peat (om_frac = 1): no unconnected conductivity
    om[30:40] = 0.6 * inputs.ORGANIC_MAX       # just above the percolation threshold
    _, zs, _ = inputs.layer_structure_20sl()
    got = inputs.pedotransfer(sand, clay, om, zs)
    for c in range(n):
        for lev in range(1, inputs.NLEVGRND + 1):
            want = restated(float(sand[c]), float(clay[c]), float(om[c]), float(zs[lev - 1]), lev)
            for k, v in want.items():
                np.testing.assert_allclose(got[k][lev - 1, c], v, rtol=1e-13, err_msg="%s c=%d lev=%d" % (k, c, lev))


def test_cosby_table5_known_values():
    """Mineral soil (om = 0) at 50 % sand, 20 % clay by hand from the pinned
    coefficients: watsat = 0.489 - 0.00126*50, bsw = 2.91 + 0.159*20,
    sucsat = 10*10^(1.88 - 0.0131*50) mm, hksat = 0.0070556*10^(-0.884 + 0.0153*50) mm/s."""
    _, zs, _ = inputs.layer_structure_20sl()
    got = inputs.pedotransfer(np.array([50.0]), np.array([20.0]), np.array([0.0]), zs)
    assert abs(got["watsat"][0, 0] - 0.426) < 1e-15
    assert abs(got["bsw"][0, 0] - 6.09) < 1e-14
    assert abs(got["sucsat"][0, 0] - 10.0 * 10.0 ** 1.225) < 1e-11
    assert abs(got["hksat"][0, 0] - 0.0070556 * 10.0 ** (-0.119)) < 1e-17
