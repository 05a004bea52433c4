"""Regenerates the golden fixtures in this directory from the reference's own
tests and technical-note tables, read as text from a checkout of the
reference whose path is the one required argument:

  layer_table_20sl.json  doc/source/tech_note/Ecosystem/CLM50_Tech_Note_Ecosystem.rst:164-219
  skip_steps.json        src/biogeophys/test/Balance_test/test_Balance.pf:40-105
  quadratic_kat.json     src/utils/test/quadratic_test/test_quadratic.pf
  qsat_coeffs.json       src/biogeophys/QSatMod.F90:16-54
  pedotransfer.json      src/main/FuncPedotransferMod.F90:28,83-103 (the default
                         Cosby 1984 table 5) and the organic-soil mixing of
                         src/biogeophys/SoilStateInitTimeConstMod.F90:200-210,543-602
  restart_vars.json      the restartvar declarations (name, type, dimensions,
                         dimension order on file) of the path's prognostic
                         state: TemperatureType.F90, WaterStateType.F90,
                         WaterStateBulkType.F90, WaterDiagnosticBulkType.F90,
                         SoilHydrologyType.F90, subgridRestMod.F90

    python tests/golden/make_golden.py <path of the reference checkout>
"""
import json
import os
import re
import sys

if len(sys.argv) != 2:
    sys.exit("usage: make_golden.py <path of the reference checkout>")
REF = sys.argv[1]
OUT = os.path.dirname(os.path.abspath(__file__))


def read(rel):
    with open(os.path.join(REF, rel)) as f:
        return f.read()


def layer_table():
    txt = read("doc/source/tech_note/Ecosystem/CLM50_Tech_Note_Ecosystem.rst")
    start = txt.index(".. _Table Soil layer structure:")
    rows = []
    for line in txt[start:].splitlines():
        m = re.match(r"\s*\|\s*(\d+)\s*\|\s*([\d.]+)\s*\|\s*([\d.]+)\s*\|\s*([\d.]+)\s*\|", line)
        if m:
            rows.append([int(m.group(1)), float(m.group(2)), float(m.group(3)), float(m.group(4))])
        if len(rows) == 25:
            break
    return {"source": "CLM50_Tech_Note_Ecosystem.rst, Table Soil layer structure",
            "columns": ["layer", "z", "dz", "zh"], "rows": rows, "decimals": 3}


def skip_steps():
    txt = read("src/biogeophys/test/Balance_test/test_Balance.pf")
    cases = []
    for block in txt.split("@Test")[1:]:
        d = re.search(r"dtime\s*=\s*(\d+)", block)
        a = re.search(r"@assertEqual\(\s*(\d+)\s*,\s*nskip", block)
        if d and a:
            cases.append([int(d.group(1)), int(a.group(1))])
    return {"source": "test_Balance.pf", "skip_size_s": 3600.0, "cases": cases}


def _arr(block, name):
    m = re.search(name + r"\s*=\s*\(/(.*?)/\)", block, re.S)
    return [float(x.replace("_r8", "").strip()) for x in m.group(1).split(",")]


def quadratic():
    txt = read("src/utils/test/quadratic_test/test_quadratic.pf")
    sub = {m.group(1): m.group(2) for m in re.finditer(r"subroutine (\w+)\(this\)(.*?)end subroutine", txt, re.S)}
    zr = sub["zero_root"]
    sr = sub["simple_roots"]
    return {
        "source": "test_quadratic.pf",
        "tol": 1e-15, "tol_big": 1e-6,
        "zero_root": {"a": _arr(zr, r"\ba"), "b": 0.0, "c": 0.0, "r1": 0.0, "r2": 1e36},
        "simple_roots": {"a": _arr(sr, r"\ba"), "b": _arr(sr, r"\bb"), "c": _arr(sr, r"\bc"),
                         "r1": _arr(sr, "expectedr1"), "r2": _arr(sr, "expectedr2")},
        "near_zero_sqrts": {"a": 1.0, "b": 4.0, "c": 4.0, "pert_eps": [0.0, 0.5, 2.0], "r1": -2.0},
        "errors": [{"a": 0.0, "b": 0.0, "c": 0.0, "msg": "quadratic ERROR: Quadratic solution error"},
                   {"a": 1.0, "b": 2.0, "c": 5.0,
                    "msg": "quadratic ERROR: Quadratic solution error: b^2 - 4ac is negative"},
                   {"a": 1.0, "b": 4.0, "c_plus_eps": 100.0,
                    "msg": "quadratic ERROR: Quadratic solution error: b^2 - 4ac is negative"}],
    }


def qsat():
    txt = read("src/biogeophys/QSatMod.F90")
    out = {}
    for name in ("a", "b", "c", "d"):
        vals = []
        for i in range(0, 9):
            m = re.search(r"\b%s%d\s*=\s*([-+0-9.eE]+)_r8" % (name, i), txt)
            if m:
                vals.append(float(m.group(1)))
        out[name] = vals
    return {"source": "QSatMod.F90 (Flatau et al. 1992 coefficients)", "coeffs": out}


def _rhs(line):
    """Right-hand side of a Fortran assignment, comment stripped, blanks squeezed."""
    return " ".join(line.split("!")[0].split("=", 1)[1].split())


def pedotransfer():
    """The expressions of the default pedotransfer function and of the
    organic-soil mixing, as the reference's source lines state them."""
    ft = read("src/main/FuncPedotransferMod.F90")
    assert re.search(r"ipedof0\s*=\s*cosby_1984_table5", ft)
    body = ft[ft.index("subroutine pedotransf_cosby1984_table5"):]
    body = body[:body.index("end subroutine pedotransf_cosby1984_table5")]
    t5 = {name: _rhs(next(l for l in body.splitlines() if re.match(r"\s*%s\s*=" % name, l)))
          for name in ("watsat", "bsw", "sucsat", "xksat")}
    st = read("src/biogeophys/SoilStateInitTimeConstMod.F90").splitlines()
    consts = {name: _rhs(next(l for l in st if re.search(r"::\s*%s\s*=" % name, l)).split("::", 1)[1])
              for name in ("zsapric", "pcalpha", "pcbeta")}
    org = {name: _rhs(next(l for l in st if re.match(r"\s*%s\s+=\s*m" % name, l)))
           for name in ("om_watsat", "om_b", "om_sucsat", "om_hksat")}

    def stmt(key, first):
        i = next(k for k, l in enumerate(st) if key in l and first in l)
        text = st[i]
        while text.split("!")[0].rstrip().endswith("&"):
            i += 1
            text = text.split("!")[0].rstrip()[:-1] + " " + st[i].strip().lstrip("&")
        return _rhs(text)
    return {"source": "FuncPedotransferMod.F90 pedotransf_cosby1984_table5; SoilStateInitTimeConstMod.F90",
            "table5": t5, "constants": consts, "organic": org,
            "tkdry": stmt("tkdry_col(c,lev)", "0.135_r8"), "tksatu": stmt("tksatu_col(c,lev)", "0.57_r8"),
            "bsw": stmt("bsw_col(c,lev)", "bsw_sf"), "watsat": stmt("watsat_col(c,lev)    =", "watsat_sf")}


RESTART_SOURCES = ("src/biogeophys/TemperatureType.F90", "src/biogeophys/WaterStateType.F90",
                   "src/biogeophys/WaterStateBulkType.F90", "src/biogeophys/WaterDiagnosticBulkType.F90",
                   "src/biogeophys/SoilHydrologyType.F90", "src/main/subgridRestMod.F90")
RESTART_NAMES = ("T_SOISNO", "T_GRND", "TH2OSFC", "T_VEG", "H2OSOI_LIQ", "H2OSOI_ICE", "H2OSFC",
                 "H2OSNO_NO_LAYERS", "WA", "ZWT", "ZWT_PERCH", "FROST_TABLE", "SNLSNO", "SNOW_DEPTH",
                 "frac_sno_eff", "frac_sno", "FH2OSFC", "INT_SNOW", "SNOMELT_ACCUM", "LIQCAN", "SNOCAN")


def _call_text(txt, start):
    """The text of a Fortran call from `start` to its closing parenthesis
    (parentheses inside quoted strings and comments do not count)."""
    i = txt.index("(", start) + 1
    depth, quote = 1, None
    while depth:
        c = txt[i]
        if quote:
            if c == quote:
                quote = None
        elif c in "'\"":
            quote = c
        elif c == "!":
            i = txt.index("\n", i)
            continue
        elif c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
        i += 1
    return txt[start:i]


def restart_vars():
    out = {}
    for rel in RESTART_SOURCES:
        txt = read(rel)
        for m in re.finditer(r"call\s+restartvar\s*\(", txt):
            call = _call_text(txt, m.start())
            flat = re.sub(r"&\s*(!.*)?\n\s*&?", " ", call)
            vm = re.search(r"varname\s*=\s*(?:this%info%fname\(\s*)?'(\w+)'", flat)
            if not vm or vm.group(1) not in RESTART_NAMES or vm.group(1) in out:
                continue
            def opt(key, pat=r"'(\w+)'"):
                r = re.search(key + r"\s*=\s*" + pat, flat)
                return r.group(1).strip() if r else None
            out[vm.group(1)] = {"file": rel, "line": txt.count("\n", 0, m.start()) + 1,
                                "xtype": opt("xtype", r"(\w+)"), "dim1name": opt("dim1name"),
                                "dim2name": opt("dim2name"), "switchdim": opt("switchdim", r"(\.\w+\.)") == ".true.",
                                "lowerb2": opt("lowerb2", r"([^,)]+)"), "upperb2": opt("upperb2", r"([^,)]+)")}
    missing = [n for n in RESTART_NAMES if n not in out]
    if missing:
        sys.exit("restartvar declarations not found: %s" % missing)
    return {"source": "restartvar calls of %s" % ", ".join(os.path.basename(r) for r in RESTART_SOURCES),
            "vars": out}


def main():
    for fname, fn in (("layer_table_20sl.json", layer_table), ("skip_steps.json", skip_steps),
                      ("quadratic_kat.json", quadratic), ("qsat_coeffs.json", qsat),
                      ("pedotransfer.json", pedotransfer), ("restart_vars.json", restart_vars)):
        with open(os.path.join(OUT, fname), "w") as f:
            json.dump(fn(), f, indent=1)
        print("wrote", fname)


if __name__ == "__main__":
    main()
