// soil_kernels.cu -- sm_103a FP64 kernels for SoilWater (Zeng-Decker 2009) and
// SoilTemperature (snow + surface water + soil + bedrock heat solve with phase
// change).  One thread owns one column; every level array is read and written
// level-major with consecutive columns in consecutive lanes, so each warp-wide
// access is one coalesced 256-byte transaction.
//
// The banded heat system is factored with a streaming form of LAPACK dgbtf2
// (partial pivoting, kl = ku = 2) that keeps a 3 x 5 window of the matrix in
// registers, folds dgbtrs' forward substitution into the factorisation, and
// stores each finished U row plus its forward-substituted right-hand side in a
// per-column slot of a device scratch buffer (6 doubles per row, rows-major,
// columns innermost).  The back substitution (dtbsv) then streams those rows
// from the bottom up.  The sequence of floating-point operations on every
// matrix and vector element is the one dgbtf2 + dgbtrs + dtbsv perform.
#include <cuda_runtime.h>
#include <cstdint>
#include "ctsm_device.cuh"
#include <mutex>
#include "soil_kernels.cuh"
#include "soil_math.cuh"
#include "cr_div.cuh"
#include "fcmp.cuh"
#include "moisture_form_device.cuh"
#include "moisture_form_kernels.cuh"
#include "hydrology_device.cuh"
#include "soilfluxes_device.cuh"
#include "capi_internal.h"

namespace ctsmg {

__device__ __forceinline__ double ipow4(double x) { double x2 = x * x; return x2 * x2; }
__device__ __forceinline__ double ipow3(double x) { double x2 = x * x; return x2 * x; }

// ============================================================ SoilWater (ZD09)
// src/biogeophys/SoilWaterMovementMod.F90:414-972 for one column, as one
// downward sweep.  Level j+1's water content, ice fraction, equilibrium
// matric potential and node potential are formed one level ahead, so row j
// of the tridiagonal system (:775-894) is complete as soon as the sweep
// reaches it and is eliminated at once (the forward pass of
// TridiagonalMod.F90:67-80); only the elimination's gam and r vectors are
// kept for the back substitution (:82-89).  Every value is the reference's
// expression on the reference's operands; quotients that share a divisor
// (the porosity, the suction, the node spacing, dtime, the pivot bet) are
// formed from one correctly rounded reciprocal (cr_div.cuh), which gives the
// same bits as the division.
struct ZdLevel {
    double zmm, dzmm, zimm, ws, bb, vwc, icef, zq, smp, dsmpdw, hks;
};

__device__ __forceinline__ ZdLevel zd09_level(const ctsmg_soilwater_io& io, int c, int j, double zimm_prev,
                                              double zwtmm, double smpmin) {
    const int ld = io.ldc;
    const size_t ss_ix = c + (size_t)(j - LS) * ld, g_ix = c + (size_t)(j - 1) * ld;
    ZdLevel L;
    const double dzj = io.dz[ss_ix], ws = io.watsat[g_ix], ss = io.sucsat[g_ix], bb = io.bsw[g_ix];
    L.ws = ws;
    L.bb = bb;
    L.hks = io.hksat[g_ix];
    L.zmm = io.z[ss_ix] * 1.e3;
    L.dzmm = dzj * 1.e3;
    L.zimm = io.zi[c + (size_t)(j + NLEVSNO) * ld] * 1.e3;
    const Recip rws = recip(ws);
    // :649-665 ice fraction and liquid content
    const double vol_ice = ic::min(ws, divf(io.h2osoi_ice[ss_ix], dzj * DENICE));
    L.icef = ic::minc(divr(vol_ice, rws), 1.0);
    io.icefrac[g_ix] = L.icef;
    L.vwc = divf(ic::maxc(io.h2osoi_liq[ss_ix], 1.0e-6), dzj * DENH2O);
    // :670-712 equilibrium volumetric water and matric potential: water table
    // above the layer, inside it, below it.  temp0 is the same expression in
    // the last two cases and tempi is only needed in the last, so each power
    // has one call site.
    const bool above = ic::le(zwtmm, zimm_prev);
    const bool inside = !above && ic::lt(zwtmm, L.zimm) && ic::gt(zwtmm, zimm_prev);
    double temp0 = 0.0, tempi = 1.0, veq, omb = 0.0;
    if (!above) {
        const Recip rss = recip(ss);
        omb = 1.0 - divf(1.0, bb);                // 1 - 1/b
        temp0 = fm::pow(divr(ss + zwtmm - zimm_prev, rss), omb);
        if (!inside) tempi = fm::pow(divr(ss + zwtmm - L.zimm, rss), omb);
    }
    if (above) {
        veq = ws;
    } else if (inside) {
        double voleq1 = divf(divf(-ss * ws, omb), zwtmm - zimm_prev) * (tempi - temp0);
        veq = divf(voleq1 * (zwtmm - zimm_prev) + ws * (L.zimm - zwtmm), L.zimm - zimm_prev);
        veq = ic::min(ws, veq);
        veq = ic::max0(veq);
    } else {
        veq = divf(divf(-ss * ws, omb), L.zimm - zimm_prev) * (tempi - temp0);
        veq = ic::max0(veq);
        veq = ic::min(ws, veq);
    }
    L.zq = ic::max(smpmin, -ss * fm::pow(ic::maxc(divr(veq, rws), 0.01), -bb));
    // :740-760 node matric potential and its derivative
    double s_node = ic::maxc(divr(L.vwc, rws), 0.01);
    s_node = ic::minc(s_node, 1.0);
    const double sm = ic::max(smpmin, -ss * fm::pow(s_node, -bb));
    L.smp = sm;
    L.dsmpdw = divf(-bb * sm, L.vwc);
    io.smp_l[g_ix] = sm;
    return L;
}

__device__ void zd09_column(const ctsmg_soilwater_io& io, int c, double e_ice, double dtime) {
    const int ld = io.ldc;
    auto SS = [&](const double* p, int j) { return p[c + (size_t)(j - LS) * ld]; };
    auto G = [&](const double* p, int j) { return p[c + (size_t)(j - 1) * ld]; };
    auto ZI = [&](int j) { return io.zi[c + (size_t)(j + NLEVSNO) * ld]; };
    auto ROOT = [&](int j) { return io.qflx_rootsoi[c + (size_t)(j - 1) * ld]; };
    auto setq = [&](int j, double qi, double qo) {
        io.qin[c + (size_t)(j - 1) * ld] = qi;
        io.qout[c + (size_t)(j - 1) * ld] = qo;
    };

    const double zwt = io.zwt[c], smpmin = io.smpmin[c];
    const double zwtmm = zwt * 1.e3;
    const Recip rdt = recip(dtime);

    // :638-647 index of the layer right above the water table
    int jwt = NLEVSOI;
#pragma unroll 1
    for (int j = 1; j <= NLEVSOI; ++j) {
        if (ic::le(zwt, ZI(j))) { jwt = j - 1; break; }
    }
    // :649-665 water content at the water table (frozen case)
    double vwc_zwt = G(io.watsat, NLEVSOI);
    if (ic::ltc(SS(io.t_soisno, jwt + 1), TFRZ)) {
        vwc_zwt = fmax(SS(io.h2osoi_liq, NLEVSOI), 1.0e-6) / (SS(io.dz, NLEVSOI) * DENH2O);
#pragma unroll 1
        for (int j = NLEVSOI; j <= NLEVGRND; ++j) {
            if (zwt <= ZI(j)) {
                const double t = SS(io.t_soisno, j);
                double smp1 = HFUS * (TFRZ - t) / (GRAV * t) * 1000.0;
                smp1 = fmax(G(io.sucsat, NLEVSOI), smp1);
                vwc_zwt = G(io.watsat, NLEVSOI) * fm::pow(smp1 / G(io.sucsat, NLEVSOI), -1.0 / G(io.bsw, NLEVSOI));
                vwc_zwt = fmin(vwc_zwt, sp(0.5f) * (G(io.watsat, NLEVSOI) + G(io.h2osoi_vol, NLEVSOI)));
                break;
            }
        }
    }

    // forward elimination state: gam(j) and the eliminated right-hand side
    // r(j) per row, bet of the last row and its reciprocal, c of the last row
    constexpr int N1 = NLEVSOI + 2;
    double gam[N1], rr[N1];
    Recip rbet{};
    double c_prev = 0.0;
    auto eliminate = [&](int j, double a, double b, double cc, double r) {
        if (j == 1) {
            rbet = recip(b);
            rr[1] = divr(r, rbet);
        } else {
            const double g = divr(c_prev, rbet);
            const double bet = b - a * g;
            rbet = recip(bet);
            rr[j] = divr(r - a * rr[j - 1], rbet);
            gam[j] = g;
        }
        c_prev = cc;
    };

    // values the recharge needs (:919-955): imped at jwt+1, smp and zq at max(1, jwt)
    const int jq = jwt + 1, jm = max(1, jwt);
    double imped_q = 0.0, smp_m = 0.0, zq_m = 0.0;

    ZdLevel cur = zd09_level(io, c, 1, 0.0, zwtmm, smpmin);
    double q_up = 0.0, dq_up0 = 0.0, dq_up1 = 0.0;
#pragma unroll 1
    for (int j = 1; j <= NLEVSOI; ++j) {
        const bool bottom = j == NLEVSOI;
        ZdLevel nx = bottom ? cur : zd09_level(io, c, j + 1, cur.zimm, zwtmm, smpmin);
        // :716-737 interface conductivity and its derivative (jp = min(nlevsoi, j+1))
        const Recip rB = recip(cur.ws + nx.ws);
        const double s1 = ic::minc(divr(cur.vwc + nx.vwc, rB), 1.0);
        const double s2 = cur.hks * fm::pow(s1, 2.0 * cur.bb + 2.0);
        const double imped = pow10_dd(-e_ice * (0.5 * (cur.icef + nx.icef)));
        const double hk = imped * s1 * s2;
        const double dhkdw = imped * (2.0 * cur.bb + 3.0) * s2 * divr(1.0, rB);
        io.hk_l[c + (size_t)(j - 1) * ld] = hk;
        if (j == jq) imped_q = imped;
        if (j == jm) { smp_m = cur.smp; zq_m = cur.zq; }
        if (!bottom) {
            // :775-846 top and interior rows; the inflow of level j and its
            // derivatives are the outflow of level j-1 and its derivatives
            const Recip rden = recip(nx.zmm - cur.zmm);
            const double num = (nx.smp - cur.smp) - (nx.zq - cur.zq);
            const double qout = divr(-hk * num, rden);
            const double dqodw1 = divr(-(-hk * cur.dsmpdw + num * dhkdw), rden);
            const double dqodw2 = divr(-(hk * nx.dsmpdw + num * dhkdw), rden);
            if (j == 1) {
                const double qin = io.qflx_infl[c];
                eliminate(1, 0.0, cur.dzmm * (0.0 + divr(1.0, rdt)) + dqodw1, dqodw2, qin - qout - ROOT(1));
                setq(1, qin, qout);
            } else {
                eliminate(j, -dq_up0, divr(cur.dzmm, rdt) - dq_up1 + dqodw1, dqodw2, q_up - qout - ROOT(j));
                setq(j, q_up, qout);
            }
            q_up = qout; dq_up0 = dqodw1; dq_up1 = dqodw2;
        } else {
            // :847-894 bottom node and the aquifer layer below it
            const double zmm_a = sp(0.5f) * (1.e3 * zwt + cur.zmm);
            const double dzmm_a = (jwt < NLEVSOI) ? cur.dzmm : (1.e3 * zwt - cur.zmm);
            if (j > jwt) {
                eliminate(j, -dq_up0, divr(cur.dzmm, rdt) - dq_up1 + 0.0, 0.0, q_up - 0.0 - ROOT(j));
                setq(j, q_up, 0.0);
                eliminate(j + 1, 0.0, divr(dzmm_a, rdt), 0.0, 0.0);
            } else {
                // zq of the aquifer node (:701-712)
                const double ss = G(io.sucsat, j), ws = cur.ws, bb = cur.bb;
                const double tempi = 1.0;
                const double temp0 = fm::pow(((ss + zwtmm - cur.zimm) / ss), 1.0 - 1.0 / bb);
                double veq = -ss * ws / (1.0 - 1.0 / bb) / (zwtmm - cur.zimm) * (tempi - temp0);
                veq = fmax(veq, 0.0);
                veq = fmin(ws, veq);
                const double zq_a = fmax(smpmin, -ss * fm::pow(fmax(veq / ws, 0.01), -bb));
                double s_node = fmax(sp(0.5f) * ((vwc_zwt + cur.vwc) / ws), 0.01);
                s_node = fmin(1.0, s_node);
                double smp1 = -ss * fm::pow(s_node, -bb);
                smp1 = fmax(smpmin, smp1);
                const double dsmpdw1 = -bb * smp1 / (s_node * ws);
                const Recip rden = recip(zmm_a - cur.zmm);
                const double num = (smp1 - cur.smp) - (zq_a - cur.zq);
                const double qout = divr(-hk * num, rden);
                const double dqodw1 = divr(-(-hk * cur.dsmpdw + num * dhkdw), rden);
                const double dqodw2 = divr(-(hk * dsmpdw1 + num * dhkdw), rden);
                eliminate(j, -dq_up0, divr(cur.dzmm, rdt) - dq_up1 + dqodw1, dqodw2, q_up - qout - ROOT(j));
                // the aquifer layer's inflow derivatives are dqodw1 / dqodw2
                eliminate(j + 1, -dqodw1, divr(dzmm_a, rdt) - dqodw2 + 0.0, 0.0, qout - 0.0);
                setq(j, q_up, qout);
            }
            rr[0] = dzmm_a;   // the aquifer layer's thickness, kept for the recharge
        }
        cur = nx;
    }
    // :82-89 back substitution; the solution (dwat2) overwrites r
    const double dzmm_a = rr[0];
#pragma unroll 1
    for (int j = NLEVSOI; j >= 1; --j) rr[j] = rr[j] - gam[j + 1] * rr[j + 1];
    // :912-917 update and deficit
    double deficit = 0.0;
#pragma unroll 1
    for (int j = 1; j <= NLEVSOI; ++j) {
        double& liq = io.h2osoi_liq[c + (size_t)(j - LS) * ld];
        double v = liq + rr[j] * (SS(io.dz, j) * 1.e3);
        liq = v;
        if (ic::lt0(v)) deficit = deficit - v;
    }
    double qcharge;
    if (jwt < NLEVSOI) {
        double s_node = fmax(G(io.h2osoi_vol, jq) / G(io.watsat, jq), 0.01);
        double s1 = fmin(1.0, s_node);
        double ka = imped_q * G(io.hksat, jq) * fm::pow(s1, 2.0 * G(io.bsw, jq) + 3.0);
        double smp1 = fmax(smpmin, smp_m);
        double wh = smp1 - zq_m;
        if (jwt == 0) qcharge = -ka * (0.0 - wh) / ((zwt + sp(1.e-3f)) * 1000.0);
        else qcharge = -ka * (0.0 - wh) / ((zwt - SS(io.z, jwt)) * 1000.0 * sp(2.0f));
        qcharge = fmax(-divr(10.0, rdt), qcharge);
        qcharge = fmin(divr(10.0, rdt), qcharge);
    } else {
        qcharge = divr(rr[NLEVSOI + 1] * dzmm_a, rdt);
    }
    io.qcharge[c] = qcharge;
    io.qflx_deficit[c] = deficit;
}

// ============================================================ SoilTemperature
// The band LU's tests on the integer pipe (FP64 instructions are the step's
// limit on GB300): x != 0.0 (NaN counts as nonzero, as in IEEE), and |a| > |b|
// with a NaN a or b false, as the IEEE comparison of fabs values.
__device__ __forceinline__ bool nonzero(double x) { return (__double_as_longlong(x) << 1) != 0; }
__device__ __forceinline__ unsigned long long abs_bits(double x) {
    return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}
__device__ __forceinline__ bool abs_gt(unsigned long long ua, unsigned long long ub) {
    return ua <= 0x7ff0000000000000ull && ub <= 0x7ff0000000000000ull && ua > ub;
}

// Scratch slot of one column: row i (1-based, i = 1..n) occupies 6 doubles
// U(i,i..i+4), y(i) at ws[((i-1)*6 + k) * ws_ld + slot].
struct Scratch {
    double* ws; int ld; int slot;
    __device__ __forceinline__ double& at(int i, int k) const {
        return ws[((size_t)(i - 1) * 6 + k) * ld + slot];
    }
};

// src/biogeophys/SoilTemperatureMod.F90:92-508 (and the routines it calls) for
// one natural-vegetation column.  Returns the dgbsv info (0 = success).
__device__ int soiltemp_column(const ctsmg_soiltemp_io& io, int c, int begp, double dtime,
                               int snow_method, const Scratch& S) {
    const int ld = io.ldc;
    auto ssi = [&](int j) { return c + (size_t)(j - LS) * ld; };
    auto gi = [&](int j) { return c + (size_t)(j - 1) * ld; };
    auto Z = [&](int j) { return io.z[ssi(j)]; };
    auto ZI = [&](int j) { return io.zi[c + (size_t)(j + NLEVSNO) * ld]; };
    auto DZ = [&](int j) { return io.dz[ssi(j)]; };
    double* __restrict__ T = io.t_soisno;
    double* __restrict__ LIQ = io.h2osoi_liq;
    double* __restrict__ ICE = io.h2osoi_ice;

    const int snl = io.snl[c];
    const int nbedrock = io.nbedrock[c];
    const double frac_sno = io.frac_sno_eff[c];
    const double frac_h2osfc = io.frac_h2osfc[c];
    const double emg = io.emg[c];

    constexpr int NL = NLEVSNO + NLEVGRND + 2;
    auto L = [](int j) { return j + NLEVSNO; };
    // per level: interface conductivity tk(j), diffusion factor fact(j),
    // heat flux fn(j) and the reciprocal of the node spacing z(j+1) - z(j)
    // (shared by fn, the matrix rows of levels j and j+1 and the flux from
    // the new temperatures)
    double tk[NL], fact[NL], fn[NL], rdz[NL];
    const Recip R_DENH2O = CTSMG_CONST_RECIP(DENH2O), R_DENICE = CTSMG_CONST_RECIP(DENICE);
    const Recip R_HFUS = CTSMG_CONST_RECIP(HFUS);
    const Recip rdt = recip(dtime);
    const Recip rfsno = recip(frac_sno);
    auto RDZ = [&](int j) { return Recip{Z(j + 1) - Z(j), rdz[L(j)], crdiv_in_range(Z(j + 1) - Z(j))}; };

    // ---------------- SoilThermProp (:664-896) -> thk, tk, cv, and
    // ComputeHeatDiffFluxAndFactor (:1876-1906) -> fact, fn, one level behind
    // the conductivity (fn(j) needs tk(j), which needs thk(j+1))
    double thk_prev = 0.0;
#pragma unroll 1
    for (int j = snl + 1; j <= NLEVGRND; ++j) {
        double t, cv;
        if (j >= 1) {
            const double liq = LIQ[ssi(j)], ice = ICE[ssi(j)], dzj = DZ(j), ws = io.watsat[gi(j)];
            if (j > nbedrock) {
                // the reference evaluates the soil formula here too and then
                // overwrites it with thk_bedrock (:710-725); the value is unused
                t = THK_BEDROCK;
            } else {
                double satw = divf(divr(liq, R_DENH2O) + divr(ice, R_DENICE) + 0.0 / DENICE, dzj * ws);
                satw = ic::minc(satw, 1.0);
                if (ic::gtc(satw, .1e-6)) {
                    double dke = ic::gec(T[ssi(j)], TFRZ) ? ic::max0(fm::log10(satw) + 1.0) : satw;
                    const double xl = divf(liq, DENH2O * dzj);
                    double fl = divf(xl, xl + divf(ice, DENICE * dzj) + zero_over(DENICE * dzj));
                    double dksat = io.tkmg[gi(j)] * tkwat_tkice_pow(fl * ws, (1.0 - fl) * ws);
                    t = dke * dksat + (1.0 - dke) * io.tkdry[gi(j)];
                } else {
                    t = io.tkdry[gi(j)];
                }
            }
            cv = io.csol[gi(j)] * (1.0 - ws) * dzj + (ice * CPICE + liq * CPLIQ) + 0.0 * CPICE;
            if (j > nbedrock) cv = CSOL_BEDROCK * dzj;
            if (j == 1 && ic::gt0(io.h2osno_no_layers[c])) cv = cv + CPICE * io.h2osno_no_layers[c];
        } else {
            const double liq = LIQ[ssi(j)], ice = ICE[ssi(j)];
            double b = divf(ice + liq, frac_sno * DZ(j));
            io.bw[ssi(j)] = b;
            if (snow_method == 0) {
                t = TKAIR + (7.75e-5 * b + 1.105e-6 * b * b) * (TKICE - TKAIR);
            } else {
                if (ic::lec(b, 156.0)) t = sp(0.023f) + sp(0.234f) * (b / 1000);
                else t = sp(0.138f) - sp(1.01f) * (b / 1000) + (sp(3.233f) * ((b / 1000) * (b / 1000)));
            }
            cv = ic::gt0(frac_sno) ? ic::maxc(divr(CPLIQ * liq + CPICE * ice, rfsno), THIN_SFCLAYER) : THIN_SFCLAYER;
        }
        io.thk[ssi(j)] = t;
        double f;
        if (j == snl + 1) f = divf(divf(dtime, cv) * DZ(j), 0.5 * (Z(j) - ZI(j - 1) + CAPR * (Z(j + 1) - ZI(j - 1))));
        else f = divf(dtime, cv);
        fact[L(j)] = f;
        io.fact[ssi(j)] = f;
        if (j > snl + 1) {
            const int jm = j - 1;
            const double tkm = divf(thk_prev * t * (Z(j) - Z(jm)), thk_prev * (Z(j) - ZI(jm)) + t * (ZI(jm) - Z(jm)));
            tk[L(jm)] = tkm;
            const Recip r = recip(Z(j) - Z(jm));
            rdz[L(jm)] = r.y;
            fn[L(jm)] = divr(tkm * (T[ssi(j)] - T[ssi(jm)]), r);
        }
        thk_prev = t;
    }
    tk[L(NLEVGRND)] = 0.0;
    fn[L(NLEVGRND)] = io.eflx_bot[c];
    const double thk1 = io.thk[ssi(1)];
    const double z1 = Z(1);
    double tk_h2osfc;
    {
        double zh2osfc = sp(1.0e-3f) * (sp(0.5f) * io.h2osfc[c]);
        tk_h2osfc = TKWAT * thk1 * (z1 + zh2osfc) / (TKWAT * z1 + thk1 * zh2osfc);
    }

    // ---------------- ComputeGroundHeatFluxAndDeriv (:1655-1792)
    const double t_grnd = io.t_grnd[c];
    const double t_top0 = T[ssi(snl + 1)], t_soi1 = T[ssi(1)], t_h2osfc0 = io.t_h2osfc[c];
    const double lwrad_emit = emg * SB * ipow4(t_grnd);
    const double dlwrad_emit = 4.0 * emg * SB * ipow3(t_grnd);
    const double lwrad_emit_snow = emg * SB * ipow4(t_top0);
    const double lwrad_emit_soil = emg * SB * ipow4(t_soi1);
    const double lwrad_emit_h2osfc = emg * SB * ipow4(t_h2osfc0);
    const int p0 = io.col_patchi[c] - begp, np = io.col_npatches[c];
    const double forc_lwrad = io.forc_lwrad[c], htvp = io.htvp[c];
    const int lyr_top = snl + 1;
    double hs_soil = 0.0, hs_h2osfc = 0.0, dhsdT = 0.0, hs_top_snow = 0.0;
#pragma unroll 1
    for (int p = p0; p < p0 + np; ++p) {
        const double fv = fm::i2d(io.frac_veg_nosno[p]);
        const double dl = io.dlrad[p], lw = (1.0 - fv) * emg * forc_lwrad;
        double gnet = io.sabg[p] + dl + lw - lwrad_emit - (io.eflx_sh_grnd[p] + io.qflx_evap_soi[p] * htvp);
        io.eflx_gnet[p] = gnet;
        io.sabg_chk[p] = frac_sno * io.sabg_snow[p] + (1.0 - frac_sno) * io.sabg_soil[p];
        double gsoil = io.sabg_soil[p] + dl + lw - lwrad_emit_soil - (io.eflx_sh_soil[p] + io.qflx_ev_soil[p] * htvp);
        double gh2o = io.sabg_soil[p] + dl + lw - lwrad_emit_h2osfc - (io.eflx_sh_h2osfc[p] + io.qflx_ev_h2osfc[p] * htvp);
        double dg = -io.cgrnd[p] - dlwrad_emit;
        io.dgnetdT[p] = dg;
        const double w = io.wtcol[p];
        dhsdT = dhsdT + dg * w;
        hs_soil = hs_soil + gsoil * w;
        hs_h2osfc = hs_h2osfc + gh2o * w;
    }
#pragma unroll 1
    for (int p = p0; p < p0 + np; ++p) {
        const double fv = fm::i2d(io.frac_veg_nosno[p]);
        const double w = io.wtcol[p];
        const double* sl = io.sabg_lyr;
        const size_t ldp = io.ldp;
        double stop = sl[p + (size_t)(lyr_top - LS) * ldp];
        double gsnow = stop + io.dlrad[p] + (1.0 - fv) * emg * forc_lwrad - lwrad_emit_snow -
                       (io.eflx_sh_snow[p] + io.qflx_ev_snow[p] * htvp);
        hs_top_snow = hs_top_snow + gsnow * w;
    }
    // sabg_lyr_col for levels lyr_top..1 is summed per level over patches when
    // the RHS needs it (same order of summation as the reference's patch loop)
    auto sabg_lyr_col = [&](int j) {
        double s = 0.0;
        for (int p = p0; p < p0 + np; ++p)
            s = s + io.sabg_lyr[p + (size_t)(j - LS) * io.ldp] * io.wtcol[p];
        return s;
    };

    double c_h2osfc, dz_h2osfc;
    if ((io.h2osfc[c] > THIN_SFCLAYER) && (frac_h2osfc > THIN_SFCLAYER)) {
        c_h2osfc = fmax(THIN_SFCLAYER, CPLIQ * io.h2osfc[c] / frac_h2osfc);
        dz_h2osfc = fmax(THIN_SFCLAYER, sp(1.0e-3f) * io.h2osfc[c] / frac_h2osfc);
    } else {
        c_h2osfc = THIN_SFCLAYER;
        dz_h2osfc = THIN_SFCLAYER;
    }
    io.c_h2osfc[c] = c_h2osfc;
    const double dzm_ssw = (sp(0.5f) * dz_h2osfc + z1);
    const double fn_h2osfc = tk_h2osfc * (t_soi1 - t_h2osfc0) / dzm_ssw;

    // ---------------- matrix row + RHS generator (SetRHSVec* :1913-2353,
    // SetMatrix* :2356-2926).  Row r: -nlevsno..nlevgrnd; returns the five
    // bands B(1..5, r) (band k couples row r to row r + 3 - k) and rhs(r).
    // Rows are generated once each, in ascending order.  A row's quotient
    // tk(j)/dzp is the next row's tk(j-1)/dzm (the same operands: dzm of row
    // j+1 is Z(j+1)-Z(j)), so it is carried from one row to the next (q_dn of
    // row q_row); and -(1-cnfac) fj tk / dz is the exact negation of
    // (1-cnfac) fj tk / dz.  The quotients by the node spacings use the
    // reciprocals formed with the fluxes (rdz).
    double q_dn = 0.0;
    int q_row = -1000;
    auto make_row = [&](int r, double* bnd, double& rhs) {
        bnd[0] = bnd[1] = bnd[2] = bnd[3] = bnd[4] = 0.0;
        if (r < 0) {                                   // snow layer j = r + 1
            const int j = r + 1;
            const double fj = fact[L(j)], tj = T[ssi(j)];
            if (j == snl + 1) {
                const double x = divr((1.0 - CNFAC) * fj * tk[L(j)], RDZ(j));
                bnd[2] = 1.0 + x - fj * dhsdT;
                rhs = tj + fj * (hs_top_snow - dhsdT * tj + CNFAC * fn[L(j)]);
                if (j != 0) bnd[1] = -x;
                else bnd[0] = -x;
            } else {
                bnd[3] = divr(-(1.0 - CNFAC) * fj * tk[L(j - 1)], RDZ(j - 1));
                const double qp = divr(tk[L(j)], RDZ(j));
                const double qm = (q_row == j - 1) ? q_dn : divr(tk[L(j - 1)], RDZ(j - 1));
                bnd[2] = 1.0 + (1.0 - CNFAC) * fj * (qp + qm);
                q_dn = qp;
                q_row = j;
                double rr = tj + CNFAC * fj * (fn[L(j)] - fn[L(j - 1)]);
                rhs = rr + fj * sabg_lyr_col(j);
                if (j != 0) bnd[1] = divr(-(1.0 - CNFAC) * fj * tk[L(j)], RDZ(j));
                else bnd[0] = divr(-(1.0 - CNFAC) * fj * tk[L(j)], RDZ(j));
            }
        } else if (r == 0) {                           // standing surface water
            bnd[2] = 1.0 + (1.0 - CNFAC) * (dtime / c_h2osfc) * tk_h2osfc / dzm_ssw - (dtime / c_h2osfc) * dhsdT;
            bnd[1] = -(1.0 - CNFAC) * (dtime / c_h2osfc) * tk_h2osfc / dzm_ssw;
            rhs = t_h2osfc0 + (dtime / c_h2osfc) * (hs_h2osfc - dhsdT * t_h2osfc0 + CNFAC * fn_h2osfc);
        } else {                                       // soil / bedrock layer j = r
            const int j = r;
            const double fj = fact[L(j)], tj = T[ssi(j)];
            if (j == snl + 1) {
                const double x = divr((1.0 - CNFAC) * fj * tk[L(j)], RDZ(j));
                bnd[2] = 1.0 + x - fj * dhsdT;
                bnd[1] = -x;
                rhs = tj + fj * (hs_top_snow - dhsdT * tj + CNFAC * fn[L(j)]);
            } else if (j == 1) {
                bnd[1] = divr(-(1.0 - CNFAC) * fj * tk[L(j)], RDZ(j));
                const double qp = divr(tk[L(j)], RDZ(j));
                bnd[2] = 1.0 + (1.0 - CNFAC) * fj * (qp + divr(frac_sno * tk[L(j - 1)], RDZ(j - 1))) -
                         (1.0 - frac_sno) * fj * dhsdT;
                q_dn = qp;
                q_row = j;
                bnd[4] = divr(-frac_sno * (1.0 - CNFAC) * fj * tk[L(j - 1)], RDZ(j - 1));
                double rr = tj + fj * ((1.0 - frac_sno) * (hs_soil - dhsdT * tj) + CNFAC * (fn[L(j)] - frac_sno * fn[L(j - 1)]));
                rhs = rr + frac_sno * fj * sabg_lyr_col(j);
            } else if (j <= NLEVGRND - 1) {
                bnd[1] = divr(-(1.0 - CNFAC) * fj * tk[L(j)], RDZ(j));
                const double qp = divr(tk[L(j)], RDZ(j));
                const double qm = (q_row == j - 1) ? q_dn : divr(tk[L(j - 1)], RDZ(j - 1));
                bnd[2] = 1.0 + (1.0 - CNFAC) * fj * (qp + qm);
                q_dn = qp;
                q_row = j;
                bnd[3] = divr(-(1.0 - CNFAC) * fj * tk[L(j - 1)], RDZ(j - 1));
                rhs = tj + CNFAC * fj * (fn[L(j)] - fn[L(j - 1)]);
            } else {
                const double x = divr((1.0 - CNFAC) * fj * tk[L(j - 1)], RDZ(j - 1));
                bnd[2] = 1.0 + x;
                bnd[3] = -x;
                rhs = tj - CNFAC * fj * fn[L(j - 1)] + fj * fn[L(j)];
            }
            if (j == 1 && frac_h2osfc != 0.0) {
                bnd[2] = bnd[2] + frac_h2osfc * ((1.0 - CNFAC) * fj * tk_h2osfc / dzm_ssw + fj * dhsdT);
                bnd[3] = -frac_h2osfc * (1.0 - CNFAC) * fj * tk_h2osfc / dzm_ssw;
                rhs = rhs - frac_h2osfc * fj * ((hs_soil - dhsdT * tj) + CNFAC * fn_h2osfc);
            }
        }
    };

    // ---------------- banded LU with partial pivoting + forward substitution
    const int jtop = snl, n = NLEVGRND - jtop + 1;
    // window W[a][b] = A(j+a, j+b), a = 0..2, b = 0..4;  rhs window y[a] = b(j+a)
    double W[3][5], y[3];
    {
        double bnd[5], rr;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            make_row(jtop + a, bnd, rr);
            // row i = 1 + a: A(i, i-2..i+2) = bands 5,4,3,2,1 ; window col b = i + (b - a) - 1
#pragma unroll
            for (int b = 0; b < 5; ++b) {
                const int off = b - a;            // column offset from the row's diagonal
                W[a][b] = (off >= -2 && off <= 2) ? bnd[2 - off] : 0.0;
            }
            y[a] = rr;
        }
    }
    int info = 0;
#pragma unroll 1
    for (int j = 1; j <= n; ++j) {
        const int km = min(2, n - j);
        int jp = 0;
        unsigned long long dmax = abs_bits(W[0][0]);
        if (km >= 1 && abs_gt(abs_bits(W[1][0]), dmax)) { jp = 1; dmax = abs_bits(W[1][0]); }
        if (km >= 2 && abs_gt(abs_bits(W[2][0]), dmax)) { jp = 2; }
        if (jp == 1) {
#pragma unroll
            for (int b = 0; b < 5; ++b) { double t = W[0][b]; W[0][b] = W[1][b]; W[1][b] = t; }
            double t = y[0]; y[0] = y[1]; y[1] = t;
        } else if (jp == 2) {
#pragma unroll
            for (int b = 0; b < 5; ++b) { double t = W[0][b]; W[0][b] = W[2][b]; W[2][b] = t; }
            double t = y[0]; y[0] = y[2]; y[2] = t;
        }
        if (nonzero(W[0][0])) {
            if (km > 0) {
                const double rp = divf(1.0, W[0][0]);
                W[1][0] = W[1][0] * rp;
                if (km > 1) W[2][0] = W[2][0] * rp;
#pragma unroll
                for (int b = 1; b < 5; ++b) {
                    const double yk = W[0][b];
                    if (nonzero(yk)) {
                        const double temp = -1.0 * yk;
                        W[1][b] = W[1][b] + W[1][0] * temp;
                        if (km > 1) W[2][b] = W[2][b] + W[2][0] * temp;
                    }
                }
            }
        } else if (info == 0) {
            info = j;
        }
        // dgbtrs forward step j (no-op for j = n)
        if (j < n && nonzero(y[0])) {
            const double temp = -1.0 * y[0];
            y[1] = y[1] + W[1][0] * temp;
            if (km > 1) y[2] = y[2] + W[2][0] * temp;
        }
        // finished row j -> scratch
#pragma unroll
        for (int b = 0; b < 5; ++b) S.at(j, b) = W[0][b];
        S.at(j, 5) = y[0];
        // shift the window down one row / right one column
#pragma unroll
        for (int b = 0; b < 4; ++b) { W[0][b] = W[1][b + 1]; W[1][b] = W[2][b + 1]; }
        W[0][4] = 0.0; W[1][4] = 0.0;
        y[0] = y[1]; y[1] = y[2];
        if (j + 3 <= n) {
            double bnd[5], rr;
            make_row(jtop + j + 2, bnd, rr);
            // row j+3 in window cols j+1..j+5: offsets -2..+2
            W[2][0] = bnd[4]; W[2][1] = bnd[3]; W[2][2] = bnd[2];
            W[2][3] = (j + 4 <= n) ? bnd[1] : 0.0;
            W[2][4] = (j + 5 <= n) ? bnd[0] : 0.0;
            y[2] = rr;
        } else {
#pragma unroll
            for (int b = 0; b < 5; ++b) W[2][b] = 0.0;
            y[2] = 0.0;
        }
    }
    if (info != 0) return info;

    // ---------------- dtbsv: back substitution, x(i) overwrites y(i)
    // window x[k] = x(j - k), k = 0..4 (x(j) final once divided)
    double x[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) x[k] = (n - k >= 1) ? S.at(n - k, 5) : 0.0;
#pragma unroll 1
    for (int j = n; j >= 1; --j) {
        if (nonzero(x[0])) {
            x[0] = divf(x[0], S.at(j, 0));
            const double temp = x[0];
#pragma unroll
            for (int k = 1; k <= 4; ++k)
                if (j - k >= 1) x[k] = x[k] - temp * S.at(j - k, k);   // U(j-k, j)
        }
        S.at(j, 5) = x[0];
#pragma unroll
        for (int k = 0; k < 4; ++k) x[k] = x[k + 1];
        x[4] = (j - 5 >= 1) ? S.at(j - 5, 5) : 0.0;
    }
    auto TV = [&](int r) { return S.at(r - jtop + 1, 5); };

    // unpack (:422-434) and fn1 (:438-483) -- fn1 needs the new temperatures
#pragma unroll 1
    for (int j = snl + 1; j <= NLEVGRND; ++j) T[ssi(j)] = TV(j <= 0 ? j - 1 : j);
    double t_h2osfc = (frac_h2osfc == 0.0) ? T[ssi(1)] : TV(0);
    io.t_h2osfc[c] = t_h2osfc;
    const double fn1_1 = divr(tk[L(1)] * (T[ssi(2)] - T[ssi(1)]), RDZ(1));
    io.eflx_fgr12[c] = -CNFAC * fn[L(1)] - (1.0 - CNFAC) * fn1_1;
#pragma unroll 1
    for (int j = 1; j <= NLEVGRND; ++j) {
        double v;
        if (j < NLEVGRND) {
            double fn1 = divr(tk[L(j)] * (T[ssi(j + 1)] - T[ssi(j)]), RDZ(j));
            v = -CNFAC * fn[L(j)] - (1.0 - CNFAC) * fn1;
        } else {
            v = 0.0;
        }
        io.eflx_fgr[gi(j)] = v;
    }

    // ---------------- PhaseChangeH2osfc (:960-1127)
    io.xmf_h2osfc[c] = 0.0;
    io.qflx_h2osfc_to_ice[c] = 0.0;
    io.eflx_h2osfc_to_snow[c] = 0.0;
    if (frac_h2osfc > 0.0 && t_h2osfc <= TFRZ) {
        double h2osno_total = io.h2osno_no_layers[c];
        for (int j = snl + 1; j <= 0; ++j) h2osno_total = h2osno_total + ICE[ssi(j)] + LIQ[ssi(j)];
        double h2osfc = io.h2osfc[c];
        double tinc = TFRZ - t_h2osfc;
        t_h2osfc = TFRZ;
        double hm = frac_h2osfc * (dhsdT * tinc - divr(tinc * c_h2osfc, rdt));
        double xm = divr(hm * dtime, R_HFUS);
        double temp1 = h2osfc + xm;
        double z_avg = frac_sno * io.snow_depth[c];
        double rho_avg = (z_avg > 0.0) ? fmin(800.0, h2osno_total / z_avg) : 200.0;
        const double fact0 = fact[L(0)];
        if (temp1 >= 0.0) {
            io.int_snow[c] = io.int_snow[c] - xm;
            if (snl == 0) io.h2osno_no_layers[c] = io.h2osno_no_layers[c] - xm;
            else ICE[ssi(0)] = ICE[ssi(0)] - xm;
            h2osno_total = h2osno_total - xm;
            io.h2osfc[c] = h2osfc + xm;
            io.xmf_h2osfc[c] = hm;
            io.qflx_h2osfc_to_ice[c] = divr(-xm, rdt);
            if (frac_sno > 0 && snl < 0) io.snow_depth[c] = h2osno_total / (rho_avg * frac_sno);
            else io.snow_depth[c] = h2osno_total / DENICE;
            if (snl == 0) {
                T[ssi(0)] = t_h2osfc;
                io.eflx_h2osfc_to_snow[c] = 0.;
            } else {
                double c1 = (snl == -1) ? frac_sno * (dtime / fact0 - dhsdT * dtime) : frac_sno / fact0 * dtime;
                double c2 = (frac_h2osfc != 0.0) ? (-CPLIQ * xm - frac_h2osfc * dhsdT * dtime) : 0.0;
                double t0 = (c1 * T[ssi(0)] + c2 * t_h2osfc) / (c1 + c2);
                T[ssi(0)] = t0;
                io.eflx_h2osfc_to_snow[c] = divr((t_h2osfc - t0) * c2, rdt);
            }
        } else {
            rho_avg = (h2osno_total * rho_avg + h2osfc * DENICE) / (h2osno_total + h2osfc);
            io.int_snow[c] = io.int_snow[c] + h2osfc;
            if (snl == 0) io.h2osno_no_layers[c] = io.h2osno_no_layers[c] + h2osfc;
            else ICE[ssi(0)] = ICE[ssi(0)] + h2osfc;
            h2osno_total = h2osno_total + h2osfc;
            io.qflx_h2osfc_to_ice[c] = divr(h2osfc, rdt);
            t_h2osfc = t_h2osfc - temp1 * HFUS / (dtime * dhsdT - c_h2osfc);
            io.xmf_h2osfc[c] = (hm - divr(frac_h2osfc * temp1 * HFUS, rdt));
            if (snl == 0) {
                T[ssi(0)] = t_h2osfc;
            } else {
                double c1 = (snl == -1) ? frac_sno * (dtime / fact0 - dhsdT * dtime) : frac_sno / fact0 * dtime;
                double c2 = (frac_h2osfc != 0.0) ? frac_h2osfc * (c_h2osfc - dtime * dhsdT) : 0.0;
                double t0 = (c1 * T[ssi(0)] + c2 * t_h2osfc) / (c1 + c2);
                T[ssi(0)] = t0;
                t_h2osfc = t0;
            }
            io.h2osfc[c] = 0.0;
            if (frac_sno > 0 && snl < 0) io.snow_depth[c] = h2osno_total / (rho_avg * frac_sno);
            else io.snow_depth[c] = h2osno_total / DENICE;
        }
        io.t_h2osfc[c] = t_h2osfc;
    }

    // ---------------- Phasechange (:1214-1527), one level at a time: the
    // identification, energy and mass updates of level j only read level j.
    double xmf = 0.0, qflx_snomelt = 0.0, qflx_snofrz = 0.0, qflx_snow_drain = 0.0;
#pragma unroll 1
    for (int j = LS; j <= 0; ++j) {
        io.qflx_snomelt_lyr[ssi(j)] = 0.0;
        io.qflx_snofrz_lyr[ssi(j)] = 0.0;
    }
#pragma unroll 1
    for (int j = snl + 1; j <= NLEVGRND; ++j) {
        const size_t ix = ssi(j);
        const double wice0 = ICE[ix], wliq0 = LIQ[ix];
        const double wmass0 = wice0 + wliq0 + 0.0;
        double tj = T[ix];
        int imelt = 0;
        double tinc = 0.0, supercool = 0.0;
        if (j <= 0) {
            if (ic::gt0(wice0) && ic::gtc(tj, TFRZ)) { imelt = 1; tinc = TFRZ - tj; tj = TFRZ; }
            if (ic::gt0(wliq0) && ic::ltc(tj, TFRZ)) { imelt = 2; tinc = TFRZ - tj; tj = TFRZ; }
        } else {
            if (ic::gt0(wice0) && ic::gtc(tj, TFRZ)) { imelt = 1; tinc = TFRZ - tj; tj = TFRZ; }
            if (ic::ltc(tj, TFRZ)) {
                double smp = divf(HFUS * (TFRZ - tj), GRAV * tj) * 1000.0;
                supercool = io.watsat[gi(j)] * fm::pow(divf(smp, io.sucsat[gi(j)]), divf(-1.0, io.bsw[gi(j)]));
                supercool = supercool * DZ(j) * 1000.0;
            }
            if (ic::gt(wliq0, supercool) && ic::ltc(tj, TFRZ)) { imelt = 2; tinc = TFRZ - tj; tj = TFRZ; }
            if (j == 1 && ic::gt0(io.h2osno_no_layers[c])) {
                if (ic::gtc(tj, TFRZ)) { imelt = 1; tinc = TFRZ - tj; tj = TFRZ; }
            }
        }
        const double fj = fact[L(j)];
        double hm = 0.0;
        if (imelt > 0) {
            if (j == snl + 1) {
                if (j > 0) hm = dhsdT * tinc - divf(tinc, fj);
                else hm = frac_sno * (dhsdT * tinc - divf(tinc, fj));
                if (j == 1 && frac_h2osfc != 0.0) hm = hm - frac_h2osfc * (dhsdT * tinc);
            } else if (j == 1) {
                hm = (1.0 - frac_sno - frac_h2osfc) * dhsdT * tinc - divf(tinc, fj);
            } else {
                if (j < 1) hm = -frac_sno * divf(tinc, fj);
                else hm = divf(-tinc, fj);
            }
        }
        if (imelt == 1 && ic::lt0(hm)) { hm = 0.0; imelt = 0; }
        if (imelt == 2 && ic::gt0(hm)) { hm = 0.0; imelt = 0; }
        double ice = wice0, liq = wliq0;
        if (imelt > 0 && ic::abs_gt0(hm)) {
            double xm = divr(hm * dtime, R_HFUS);
            if (j == 1) {
                if (io.h2osno_no_layers[c] > 0.0 && xm > 0.0) {
                    double temp1 = io.h2osno_no_layers[c];
                    double nl = fmax(0.0, temp1 - xm);
                    io.h2osno_no_layers[c] = nl;
                    double propor = nl / temp1;
                    io.snow_depth[c] = propor * io.snow_depth[c];
                    double heatr = hm - divr(HFUS * (temp1 - nl), rdt);
                    if (heatr > 0.0) { xm = divr(heatr * dtime, R_HFUS); hm = heatr; }
                    else { xm = 0.0; hm = 0.0; }
                    qflx_snomelt = divr(fmax(0.0, (temp1 - nl)), rdt);
                    xmf = HFUS * qflx_snomelt;
                    qflx_snow_drain = qflx_snomelt;
                }
            }
            double heatr = 0.0;
            if (ic::gt0(xm)) {
                ice = ic::max0(wice0 - xm);
                if (j >= 1) heatr = hm - divr(HFUS * (0.0 - 0.0 + wice0 - ice), rdt);
                else heatr = hm - divr(HFUS * (wice0 - ice), rdt);
            } else if (ic::lt0(xm)) {
                if (j <= 0) ice = ic::min(wmass0, wice0 - xm);
                else ice = ic::lt(wmass0 - 0.0, supercool) ? 0.0 : ic::min(wmass0 - 0.0 - supercool, wice0 - xm);
                heatr = hm - divr(HFUS * (wice0 - ice), rdt);
            }
            liq = ic::max0(wmass0 - ice - 0.0);
            if (ic::abs_gt0(heatr)) {
                if (j == snl + 1) {
                    if (j == 1) tj = tj + fj * heatr / (1.0 - (1.0 - frac_h2osfc) * fj * dhsdT);
                    else tj = tj + divr(fj, rfsno) * heatr / (1.0 - fj * dhsdT);
                } else if (j == 1) {
                    tj = tj + fj * heatr / (1.0 - (1.0 - frac_sno - frac_h2osfc) * fj * dhsdT);
                } else {
                    if (j > 0) tj = tj + fj * heatr;
                    else if (ic::gt0(frac_sno)) tj = tj + divr(fj, rfsno) * heatr;
                }
                if (j <= 0) {
                    if (ic::gt0(liq * ice)) tj = TFRZ;
                }
            }
            if (j >= 1) xmf = xmf + divr(HFUS * (wice0 - ice), rdt) + zero_over(dtime);
            else xmf = xmf + divr(HFUS * (wice0 - ice), rdt);
            if (imelt == 1 && j < 1) {
                double m = divr(ic::max0(wice0 - ice), rdt);
                io.qflx_snomelt_lyr[ix] = m;
                qflx_snomelt = qflx_snomelt + m;
                io.snomelt_accum[c] = io.snomelt_accum[c] + m * dtime * 1.e-3;
            }
            if (imelt == 2 && j < 1) {
                double f = divr(ic::max0(ice - wice0), rdt);
                io.qflx_snofrz_lyr[ix] = f;
                qflx_snofrz = qflx_snofrz + f;
            }
            ICE[ix] = ice;
            LIQ[ix] = liq;
        }
        T[ix] = tj;
        io.imelt[ix] = imelt;
    }
    io.xmf[c] = xmf;
    io.qflx_snomelt[c] = qflx_snomelt;
    io.qflx_snofrz[c] = qflx_snofrz;
    io.qflx_snow_drain[c] = qflx_snow_drain;
    io.eflx_snomelt[c] = qflx_snomelt * HFUS;

    // ---------------- t_grnd (:457-477)
    double tg;
    const double ts1 = T[ssi(1)];
    if (snl < 0) {
        if (frac_h2osfc != 0.0)
            tg = frac_sno * T[ssi(snl + 1)] + (1.0 - frac_sno - frac_h2osfc) * ts1 + frac_h2osfc * io.t_h2osfc[c];
        else
            tg = frac_sno * T[ssi(snl + 1)] + (1.0 - frac_sno) * ts1;
    } else {
        if (frac_h2osfc != 0.0) tg = (1.0 - frac_h2osfc) * ts1 + frac_h2osfc * io.t_h2osfc[c];
        else tg = ts1;
    }
    io.t_grnd[c] = tg;
    return 0;
}

// ============================================================ kernels
__global__ void __launch_bounds__(128)
soilwater_kernel(ctsmg_soilwater_io io, int begc, int nfilt, const int32_t* __restrict__ filt,
                 double e_ice, double dtime) {
    const int fc = blockIdx.x * blockDim.x + threadIdx.x;
    if (fc >= nfilt) return;
    const int c = (filt ? filt[fc] : fc + 1) - begc;
    zd09_column(io, c, e_ice, dtime);
}

__global__ void __launch_bounds__(128)
soiltemp_kernel(ctsmg_soiltemp_io io, int begc, int begp, int nfilt, const int32_t* __restrict__ filt,
                double dtime, int snow_method, double* ws, int ws_ld, DevError* err) {
    const int fc = blockIdx.x * blockDim.x + threadIdx.x;
    if (fc >= nfilt) return;
    const int c = (filt ? filt[fc] : fc + 1) - begc;
    Scratch S{ws, ws_ld, fc};
    int info = soiltemp_column(io, c, begp, dtime, snow_method, S);
    if (info != 0) report_error(err, filt ? filt[fc] : fc + begc, info, CTSMG_E_SINGULAR);
}

// One model step on one column: SoilWater then SoilTemperature (ORDER 0, the
// pairing of the plain workloads), SoilTemperature then SoilWater (ORDER 1,
// the driver's order after CanopyFluxes, clm_driver.F90:900,950), or
// SoilTemperature, SoilFluxes over the column's patches and SoilWater
// (ORDER 2, clm_driver.F90:900,921,950; sf carries the SoilFluxes components
// and the temperatures saved before the step), then the between-step refresh
// of h2osoi_vol (HydrologyNoDrainageMod.F90:580,590).
template <int BLOCK, int ORDER>
__global__ void __launch_bounds__(BLOCK)
soilstep_kernel(ctsmg_soilwater_io wio, ctsmg_soiltemp_io tio, ctsmg_soilfluxes_io sf, int ncol, double e_ice,
                double dtime, int snow_method, double* ws, int ws_ld, DevError* err, const int32_t* __restrict__ filt,
                SoilStepFlags fl) {
    const int fc = blockIdx.x * BLOCK + threadIdx.x;
    if (fc >= ncol) return;
    const int c = filt ? filt[fc] - 1 : fc;     // filt: 1-based column positions (pool mode)
    Scratch S{ws, ws_ld, fc};
    if (ORDER == 0 && fl.water) {
        zd09_column(wio, c, e_ice, dtime);
        if (fl.flexcn) flexcn_column(wio, c);
    }
    int info = soiltemp_column(tio, c, 1, dtime, snow_method, S);
    if (info != 0) report_error(err, c + 1, info, CTSMG_E_SINGULAR);
    if (ORDER == 2) {
        const int p0 = sf.col_patchi[c] - 1, np = sf.col_npatches[c];
#pragma unroll 1
        for (int p = p0; p < p0 + np; ++p) soilfluxes_patch(sf, p, c, dtime);
        soilfluxes_p2c(sf, c, 1);
    }
    if (ORDER >= 1 && fl.water) {
        zd09_column(wio, c, e_ice, dtime);
        if (fl.flexcn) flexcn_column(wio, c);
    }
    if (fl.refresh) refresh_h2osoi_vol(wio, c);
}

// The Zeng-Decker SoilWater of a resident step in its own kernel, with the
// aquifer-layer hydrology around it when HYDRO: SetSoilWaterFractions,
// SaturatedExcessRunoff and the infiltration chain before SoilWater,
// WaterTable and Drainage after it (HydrologyNoDrainageMod.F90:302-359,
// HydrologyDrainageMod.F90:132-137), the flexibleCN fix and, if refresh, the
// h2osoi_vol refresh.
template <bool HYDRO>
__global__ void __launch_bounds__(128)
zd09_step_kernel(ctsmg_soilwater_io io, int ncol, double e_ice, double dtime, int flexcn, int refresh,
                 const int32_t* __restrict__ filt, HydroStepArgs hy) {
    const int fc = blockIdx.x * blockDim.x + threadIdx.x;
    if (fc >= ncol) return;
    const int c = filt ? filt[fc] - 1 : fc;
    ctsmg_soilhydrology_params hp = hy.par;
    if (HYDRO) {
        if (hy.baseflow_scalar_c) hp.baseflow_scalar = hy.baseflow_scalar_c[c];
        if (hy.fff_c) hp.fff = hy.fff_c[c];
        set_soil_water_fractions(io, c);
        hydro::saturated_excess_runoff(hy.io, c, hp.fff);
        hydro::infiltration_chain(hy.io, c, hp, dtime);
    }
    zd09_column(io, c, e_ice, dtime);
    if (flexcn) flexcn_column(io, c);
    if (HYDRO) {
        hydro::water_table(hy.io, c, hp, dtime);
        hydro::drainage(hy.io, c, hp, dtime);
    }
    if (refresh) refresh_h2osoi_vol(io, c);
}

cudaError_t launch_zd09_step(const ctsmg_soilwater_io& io, int ncol, double e_ice, double dtime, int flexcn,
                             int refresh, const int32_t* d_filt, cudaStream_t s, const HydroStepArgs* hy) {
    if (ncol <= 0) return cudaSuccess;
    if (hy)
        zd09_step_kernel<true><<<(ncol + 127) / 128, 128, 0, s>>>(io, ncol, e_ice, dtime, flexcn, refresh, d_filt, *hy);
    else
        zd09_step_kernel<false><<<(ncol + 127) / 128, 128, 0, s>>>(io, ncol, e_ice, dtime, flexcn, refresh, d_filt,
                                                                  HydroStepArgs{});
    return cudaGetLastError();
}

// Compute_EffecRootFrac_And_VertTranSink_Default
// (src/biogeophys/SoilWaterPlantSinkMod.F90:332-420): the column root water
// sink from the patches' transpiration and root fractions.
__global__ void rootsink_kernel(const int32_t* __restrict__ col_patchi, const int32_t* __restrict__ col_npatches,
                                const double* __restrict__ wtcol, const double* __restrict__ qflx_tran_veg,
                                const double* __restrict__ rootr, int ldp, double* __restrict__ qflx_rootsoi,
                                int ncol, int ldc, const int32_t* __restrict__ filt) {
    const int fc = blockIdx.x * blockDim.x + threadIdx.x;
    if (fc >= ncol) return;
    const int c = filt ? filt[fc] - 1 : fc;
    const int p0 = col_patchi[c] - 1, np = col_npatches[c];
    double temp = 0.0, tran_col = 0.0;
    for (int p = p0; p < p0 + np; ++p) temp = temp + qflx_tran_veg[p] * wtcol[p];
    tran_col = temp;
#pragma unroll 1
    for (int j = 1; j <= NLEVSOI; ++j) {
        double rc = 0.0;
        for (int p = p0; p < p0 + np; ++p) rc = rc + rootr[p + (size_t)(j - 1) * ldp] * qflx_tran_veg[p] * wtcol[p];
        if (temp != 0.0) rc = rc / temp;
        qflx_rootsoi[c + (size_t)(j - 1) * ldc] = rc * tran_col;
    }
}

// Compute_EffecRootFrac_And_VertTranSink_Default
// (src/biogeophys/SoilWaterPlantSinkMod.F90:332-420) as the drop-in: the
// column effective root fraction and the soil water sink over a column
// filter, the column transpiration from qflx_tran_veg_col or, if that is
// NULL, the wtcol-weighted patch sum.  The per-level quotient by the
// patches' weighted transpiration shares one reciprocal.
__global__ void __launch_bounds__(128)
rootsink_dropin_kernel(ctsmg_rootsink_io io, int begc, int begp, int nfilt, const int32_t* __restrict__ filt) {
    const int fc = blockIdx.x * blockDim.x + threadIdx.x;
    if (fc >= nfilt) return;
    const int c = filt[fc] - begc;
    const int p0 = io.col_patchi[c] - begp, np = io.col_npatches[c];
    const int ldc = io.ldc, ldp = io.ldp;
    double temp = 0.0;
#pragma unroll 1
    for (int p = p0; p < p0 + np; ++p) temp = temp + io.qflx_tran_veg[p] * io.wtcol[p];
    const double tcol = io.qflx_tran_veg_col ? io.qflx_tran_veg_col[c] : temp;
    const bool scale = temp != 0.0;
    const Recip rt = recip(temp);
#pragma unroll 1
    for (int j = 1; j <= NLEVSOI; ++j) {
        double rc = 0.0;
        for (int p = p0; p < p0 + np; ++p)
            rc = rc + io.rootr[p + (size_t)(j - 1) * ldp] * io.qflx_tran_veg[p] * io.wtcol[p];
        if (scale) rc = divr(rc, rt);
        io.rootr_col[c + (size_t)(j - 1) * ldc] = rc;
        io.qflx_rootsoi[c + (size_t)(j - 1) * ldc] = rc * tcol;
    }
}

cudaError_t launch_rootsink_dropin(const ctsmg_rootsink_io& io, int begc, int begp, int nfilt, const int32_t* d_filt,
                                   cudaStream_t s) {
    if (nfilt <= 0) return cudaSuccess;
    rootsink_dropin_kernel<<<(nfilt + 127) / 128, 128, 0, s>>>(io, begc, begp, nfilt, d_filt);
    return cudaGetLastError();
}

// ------------------------------------------------------------ launchers
cudaError_t launch_soilwater(const ctsmg_soilwater_io& io, int begc, int nfilt, const int32_t* d_filt,
                             double e_ice, double dtime, cudaStream_t s) {
    if (nfilt <= 0) return cudaSuccess;
    soilwater_kernel<<<(nfilt + 127) / 128, 128, 0, s>>>(io, begc, nfilt, d_filt, e_ice, dtime);
    return cudaGetLastError();
}

cudaError_t launch_soiltemp(const ctsmg_soiltemp_io& io, int begc, int begp, int nfilt, const int32_t* d_filt,
                            double dtime, int snow_method, double* ws, int ws_ld, DevError* err, cudaStream_t s) {
    if (nfilt <= 0) return cudaSuccess;
    soiltemp_kernel<<<(nfilt + 127) / 128, 128, 0, s>>>(io, begc, begp, nfilt, d_filt, dtime, snow_method,
                                                        ws, ws_ld, err);
    return cudaGetLastError();
}

static int wave_columns(const void* kernel, int block) {
    int dev = 0, sms = 0, bpsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bpsm, kernel, block, 0) != cudaSuccess)
        return 0;
    return sms * bpsm * block;
}

int soiltemp_wave_columns() {
    static const int w = wave_columns((const void*)soiltemp_kernel, 128);
    return w;
}

template <int ORDER>
static void launch_soilstep_order(const ctsmg_soilwater_io& wio, const ctsmg_soiltemp_io& tio,
                                  const ctsmg_soilfluxes_io& sf, int ncol, double e_ice, double dtime,
                                  int snow_method, double* ws, int ws_ld, DevError* err, cudaStream_t s, int block,
                                  const int32_t* filt, SoilStepFlags fl) {
    switch (block) {
        case 64:
            soilstep_kernel<64, ORDER><<<(ncol + 63) / 64, 64, 0, s>>>(wio, tio, sf, ncol, e_ice, dtime, snow_method,
                                                                       ws, ws_ld, err, filt, fl);
            break;
        case 256:
            soilstep_kernel<256, ORDER><<<(ncol + 255) / 256, 256, 0, s>>>(wio, tio, sf, ncol, e_ice, dtime,
                                                                          snow_method, ws, ws_ld, err, filt, fl);
            break;
        default:
            soilstep_kernel<128, ORDER><<<(ncol + 127) / 128, 128, 0, s>>>(wio, tio, sf, ncol, e_ice, dtime,
                                                                          snow_method, ws, ws_ld, err, filt, fl);
            break;
    }
}

cudaError_t launch_soilstep(const ctsmg_soilwater_io& wio, const ctsmg_soiltemp_io& tio, int ncol,
                            double e_ice, double dtime, int snow_method, double* ws, int ws_ld,
                            DevError* err, cudaStream_t s, int block, int order, const int32_t* filt,
                            const ctsmg_soilfluxes_io* sf, SoilStepFlags fl) {
    if (ncol <= 0) return cudaSuccess;
    if (order == 2 && !sf) return cudaErrorInvalidValue;
    const ctsmg_soilfluxes_io none{};
    const ctsmg_soilfluxes_io& f = sf ? *sf : none;
    if (order == 2) launch_soilstep_order<2>(wio, tio, f, ncol, e_ice, dtime, snow_method, ws, ws_ld, err, s, block, filt, fl);
    else if (order == 1) launch_soilstep_order<1>(wio, tio, f, ncol, e_ice, dtime, snow_method, ws, ws_ld, err, s, block, filt, fl);
    else launch_soilstep_order<0>(wio, tio, f, ncol, e_ice, dtime, snow_method, ws, ws_ld, err, s, block, filt, fl);
    return cudaGetLastError();
}

cudaError_t launch_rootsink(const int32_t* col_patchi, const int32_t* col_npatches, const double* wtcol,
                            const double* qflx_tran_veg, const double* rootr, int ldp, double* qflx_rootsoi,
                            int ncol, cudaStream_t s, int ldc, const int32_t* filt) {
    if (ncol <= 0) return cudaSuccess;
    rootsink_kernel<<<(ncol + 127) / 128, 128, 0, s>>>(col_patchi, col_npatches, wtcol, qflx_tran_veg, rootr, ldp,
                                                       qflx_rootsoi, ncol, ldc > 0 ? ldc : ncol, filt);
    return cudaGetLastError();
}

// column gather / scatter of one level-major field: dst[l*ld + i] = src[l*ld + perm[i]]
// (gather) or dst[l*ld + perm[i]] = src[l*ld + i] (scatter); esize 4 or 8 bytes.
template <typename T>
__global__ void permute_kernel(T* __restrict__ dst, const T* __restrict__ src, const int32_t* __restrict__ perm,
                               int ncol, int nlev, int scatter) {
    const long long n = (long long)ncol * nlev;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const int l = (int)(k / ncol), i = (int)(k % ncol);
        const size_t base = (size_t)l * ncol;
        if (scatter) dst[base + perm[i]] = src[base + i];
        else dst[base + i] = src[base + perm[i]];
    }
}

cudaError_t launch_permute(void* dst, const void* src, const int32_t* perm, int ncol, int nlev, int esize,
                           int scatter, cudaStream_t s) {
    const long long n = (long long)ncol * nlev;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 32) blocks = 152 * 32;
    if (esize == 8)
        permute_kernel<double><<<blocks, 256, 0, s>>>((double*)dst, (const double*)src, perm, ncol, nlev, scatter);
    else
        permute_kernel<int32_t><<<blocks, 256, 0, s>>>((int32_t*)dst, (const int32_t*)src, perm, ncol, nlev, scatter);
    return cudaGetLastError();
}

} // namespace ctsmg

// ============================================================ allocation-free SoilTemperature
// For callers that must not allocate device memory: the host model's device
// memory is owned by another runtime (an OpenACC or OpenMP-offload build of the
// Fortran host that keeps the derived types resident and budgets every byte of
// device memory itself), or the caller runs where cudaMalloc is not acceptable
// (cudaMalloc can synchronise the device, so latency-bound callers avoid it).
// Such a caller passes device pointers for every input and output and this
// entry point uses a fixed scratch array compiled into the library instead of
// allocating one.  The array is sized for NOALLOC_MAX_COLUMNS columns (6 * 38
// doubles each, 29.9 MB); every GPU that loads the library holds it until the
// process exits.
namespace ctsmg {
constexpr int NOALLOC_MAX_COLUMNS = 16384;
static __device__ __align__(256) double g_noalloc_ws[(size_t)SOILTEMP_WS_DOUBLES_PER_COL * NOALLOC_MAX_COLUMNS];
static __device__ __align__(256) DevError g_noalloc_err;

constexpr int NOALLOC_MAX_DEVICES = 64;
static std::mutex g_noalloc_mu;
static double* g_noalloc_ws_addr[NOALLOC_MAX_DEVICES];
static DevError* g_noalloc_err_addr[NOALLOC_MAX_DEVICES];

// Error levels of the allocation-free call's device checks (every record
// carries the filter position, 1-based, so records rank by position).
constexpr int NOALLOC_BAD_FILTER = -1;     // filter entry outside begc..endc
constexpr int NOALLOC_BAD_SNL = -2;        // snl outside -nlevsno..0
constexpr int NOALLOC_BAD_NBEDROCK = -3;   // nbedrock outside 1..nlevgrnd
constexpr int NOALLOC_BAD_PATCHES = -4;    // the column's patches outside begp..endp

// Same work as soiltemp_kernel, with the filter entry and the column's snl,
// nbedrock and patch range checked on the device (the caller's filter and
// arrays are in device memory, so the host cannot check them without a
// staging copy): a bad entry is recorded as CTSMG_E_ARG with its filter
// position and a level code naming the check, and that column is skipped.
__global__ void __launch_bounds__(128)
soiltemp_noalloc_kernel(ctsmg_soiltemp_io io, int begc, int endc, int begp, int endp, int nfilt,
                        const int32_t* __restrict__ filt, double dtime, int snow_method, double* ws,
                        DevError* err) {
    const int fc = blockIdx.x * blockDim.x + threadIdx.x;
    if (fc >= nfilt) return;
    const int cg = filt ? filt[fc] : begc + fc;
    if (cg < begc || cg > endc) { report_error(err, fc + 1, NOALLOC_BAD_FILTER, CTSMG_E_ARG); return; }
    const int c = cg - begc;
    const int snl = io.snl[c], nbr = io.nbedrock[c], pi = io.col_patchi[c], np = io.col_npatches[c];
    int bad = 0;
    if (snl > 0 || snl < -NLEVSNO) bad = NOALLOC_BAD_SNL;
    else if (nbr < 1 || nbr > NLEVGRND) bad = NOALLOC_BAD_NBEDROCK;
    else if (np < 0 || pi < begp || pi + np - 1 > endp) bad = NOALLOC_BAD_PATCHES;
    if (bad) { report_error(err, fc + 1, bad, CTSMG_E_ARG); return; }
    Scratch S{ws, NOALLOC_MAX_COLUMNS, fc};
    int info = soiltemp_column(io, c, begp, dtime, snow_method, S);
    if (info != 0) report_error(err, fc + 1, info, CTSMG_E_SINGULAR);
}

// Looks up the device addresses of the scratch array and the error record
// once per device, with that device current.  ctsmg_finalize clears the table
// (noalloc_forget_devices), so after a device reset the caller runs
// ctsmg_finalize and ctsmg_init and the next call looks the addresses up anew.
static int noalloc_setup(int dev, double** ws, DevError** err) {
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return set_error(CTSMG_E_UNSUPPORTED, "device ordinal beyond the allocation-free table", dev, 0);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ws_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_ws);
        if (e != cudaSuccess) return set_error(CTSMG_E_CUDA, cudaGetErrorString(e), dev, 0);
        void* q = nullptr;
        e = cudaGetSymbolAddress(&q, g_noalloc_err);
        if (e != cudaSuccess) return set_error(CTSMG_E_CUDA, cudaGetErrorString(e), dev, 0);
        g_noalloc_ws_addr[dev] = static_cast<double*>(p);
        g_noalloc_err_addr[dev] = static_cast<DevError*>(q);
    }
    *ws = g_noalloc_ws_addr[dev];
    *err = g_noalloc_err_addr[dev];
    return 0;
}

void noalloc_forget_devices() {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    for (int d = 0; d < NOALLOC_MAX_DEVICES; ++d) {
        g_noalloc_ws_addr[d] = nullptr;
        g_noalloc_err_addr[d] = nullptr;
    }
}
} // namespace ctsmg

extern "C" int32_t ctsmg_soiltemperature_noalloc(const ctsmg_bounds* bounds, int32_t num_nolakec,
                                                 const int32_t* filter_nolakec_dev,
                                                 const ctsmg_soiltemp_io* io_dev, double dtime, void* stream) {
    using namespace ctsmg;
    int snow_method = 0;
    if (!snow_method_if_init(&snow_method))
        return set_error(CTSMG_E_NOT_INIT, "ctsmg_init has not been called", 0, 0);
    if (!bounds || !io_dev) return set_error(CTSMG_E_ARG, "null bounds or io", 0, 0);
    if (bounds->endc < bounds->begc || bounds->endp < bounds->begp - 1)
        return set_error(CTSMG_E_ARG, "empty or inverted bounds", 0, 0);
    if (num_nolakec < 0) return set_error(CTSMG_E_ARG, "negative filter length", 0, 0);
    if (num_nolakec > NOALLOC_MAX_COLUMNS)
        return set_error(CTSMG_E_ARG,
                         "ctsmg_soiltemperature_noalloc: num_nolakec exceeds the built-in scratch "
                         "(16384 columns); split the filter or use ctsmg_soiltemperature",
                         num_nolakec, 0);
    if (io_dev->ldc < bounds->endc - bounds->begc + 1 || io_dev->ldp < bounds->endp - bounds->begp + 1)
        return set_error(CTSMG_E_ARG, "ldc/ldp smaller than the bounds", 0, 0);
    if (!(dtime > 0.0)) return set_error(CTSMG_E_ARG, "dtime must be positive", 0, 0);
    if (num_nolakec == 0) return 0;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(CTSMG_E_CUDA, cudaGetErrorString(e), 0, 0);
    double* ws = nullptr;
    DevError* err = nullptr;
    int rc = noalloc_setup(dev, &ws, &err);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the error record must start at "no error" (all ones) on every call
    e = cudaMemsetAsync(err, 0xff, sizeof(DevError), s);
    if (e != cudaSuccess) return set_error(CTSMG_E_CUDA, cudaGetErrorString(e), 0, 0);
    soiltemp_noalloc_kernel<<<(num_nolakec + 127) / 128, 128, 0, s>>>(
        *io_dev, bounds->begc, bounds->endc, bounds->begp, bounds->endp, num_nolakec, filter_nolakec_dev, dtime,
        snow_method, ws, err);
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTSMG_E_CUDA, cudaGetErrorString(e), 0, 0);
    DevError h;
    e = cudaMemcpyAsync(&h, err, sizeof h, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(CTSMG_E_CUDA, cudaGetErrorString(e), 0, 0);
    if (h.key == ~0ull) return 0;
    const int code = (int)(h.key & 0xff);
    const int pos = (int)(h.key >> 32), lev = (int)((h.key >> 8) & 0xffffff) - 1024;
    if (code == CTSMG_E_SINGULAR) {
        // the reference's endrun names the column: read that filter entry back
        int32_t col = bounds->begc + pos - 1;
        if (filter_nolakec_dev) {
            e = cudaMemcpyAsync(&col, filter_nolakec_dev + (pos - 1), sizeof col, cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return set_error(CTSMG_E_CUDA, cudaGetErrorString(e), 0, 0);
        }
        return set_error(code, "BandDiagonal ERROR: dgbsv returned error code", col, lev);
    }
    const char* what = lev == NOALLOC_BAD_FILTER ? "filter entry outside begc..endc (index = filter position)"
                     : lev == NOALLOC_BAD_SNL ? "snl outside -nlevsno..0 (index = filter position)"
                     : lev == NOALLOC_BAD_NBEDROCK ? "nbedrock outside 1..nlevgrnd (index = filter position)"
                     : "column patches outside begp..endp (index = filter position)";
    return set_error(code, what, pos, lev);
}
