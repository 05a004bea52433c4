"""Generate fastmath_tables.h: the breakpoint tables of the table-driven
logarithm (Tang 1990) and exponential (Tang 1989) in fastmath.cuh.

Values are computed with mpmath at 80 significant digits and written as C99
hexadecimal literals, so the header is the same on every build host.
Run from this directory:  python gen_fastmath_tables.py > fastmath_tables.h
"""
import mpmath as mp

mp.mp.dps = 80
LOG_BITS = 8          # log breakpoints F_j = 1 + j / 256, j = 0..256
EXP_BITS = 7          # exp breakpoints 2^(j / 128), j = 0..127
GRID = mp.mpf(2) ** -42   # k*LN2_HI + LOGF_HI[j] is exact on this grid


def rn(x):
    """Round an mpmath number to the nearest double."""
    return float(x)


def on_grid(x):
    return rn(mp.nint(x / GRID) * GRID)


def hx(v):
    return float(v).hex()


ln2 = mp.log(2)
LN2_HI = on_grid(ln2)
LN2_LO = rn(ln2 - mp.mpf(LN2_HI))

out = []
out.append("// fastmath_tables.h -- generated by gen_fastmath_tables.py (mpmath, 80 digits); do not edit.")
out.append("#pragma once")
out.append(f"#define CTSMG_FM_LOG_BITS {LOG_BITS}")
out.append(f"#define CTSMG_FM_EXP_BITS {EXP_BITS}")
out.append(f"#define CTSMG_FM_LN2_HI {hx(LN2_HI)}")
out.append(f"#define CTSMG_FM_LN2_LO {hx(LN2_LO)}")
n = 1 << LOG_BITS
inv, hi, lo = [], [], []
for j in range(n + 1):
    F = 1 + mp.mpf(j) / n
    lf = mp.log(F)
    h = on_grid(lf) if j < n else LN2_HI
    l = rn(lf - mp.mpf(h)) if j < n else LN2_LO
    inv.append(rn(1 / F)); hi.append(h); lo.append(l)
out.append("// 1/F_j, and ln(F_j) = HI + LO with HI on the 2^-42 grid of LN2_HI")
out.append("#define CTSMG_FM_LOG_INVF {" + ", ".join(hx(v) for v in inv) + "}")
out.append("#define CTSMG_FM_LOG_HILO {" + ", ".join(f"{{{hx(a)}, {hx(b)}}}" for a, b in zip(hi, lo)) + "}")
m = 1 << EXP_BITS
th, tl = [], []
for j in range(m):
    T = mp.mpf(2) ** (mp.mpf(j) / m)
    a = rn(T); th.append(a); tl.append(rn(T - mp.mpf(a)))
out.append("// 2^(j/128) = HI + LO")
out.append("#define CTSMG_FM_EXP_HILO {" + ", ".join(f"{{{hx(a)}, {hx(b)}}}" for a, b in zip(th, tl)) + "}")
L = ln2 / m
L1 = rn(L); L2 = rn(L - mp.mpf(L1))
out.append(f"#define CTSMG_FM_EXP_INVL {hx(rn(m / ln2))}   // 128 / ln 2")
out.append(f"#define CTSMG_FM_EXP_L1 {hx(L1)}   // ln 2 / 128 = L1 + L2")
out.append(f"#define CTSMG_FM_EXP_L2 {hx(L2)}")
il10 = 1 / mp.log(10)
a = rn(il10)
out.append(f"#define CTSMG_FM_INV_LN10_HI {hx(a)}   // 1 / ln 10 = HI + LO")
out.append(f"#define CTSMG_FM_INV_LN10_LO {hx(rn(il10 - mp.mpf(a)))}")
print("\n".join(out))
