// ctsm_oracle_canopy.cpp -- CPU oracle (test infrastructure only) for
// CanopyFluxes + FrictionVelocity + QSat + Photosynthesis.
//
// A plain C++ restatement of the reference routines, patch by patch (the
// reference's filter compaction removes converged patches from the loop; each
// patch's own sequence of operations is unchanged by it).  Built with
// -ffp-contract=off; Fortran integer powers x**3 / x**4 are the square-and-
// multiply chains gfortran emits.  Parity for these outputs is unpinned: the
// reference has no test of CanopyFluxes or Photosynthesis-Ci; the quadratic
// solver is pinned against test_quadratic.pf and QSat's coefficients against
// the technical note.
#include <cmath>
#include <cstdint>
#include <algorithm>
#include <vector>
#include "ctsm_gpu.h"
#include "ctsm_oracle.h"
#include "oracle_libm.h"
#include "rootfind_testfns.h"

using oracle_libm::o_pow;
using oracle_libm::o_exp;
using oracle_libm::o_log;
using oracle_libm::o_atan;

namespace {

// tools/mksurfdata_esmf/src/shr_const_mod.F90:14-56, src/main/clm_varcon.F90
const double PI = 3.14159265358979323846;
const double GRAV = 9.80616;
const double SB = 5.67e-8;
const double VKC = 0.4;
const double TFRZ = 273.15;
const double CPAIR = 1.00464e3;
const double HVAP = 2.501e6;
const double RGAS = 6.02214e26 * 1.38065e-23;
const double NU_PARAM = 1.5e-5;          // clm_varcon.F90:163
const double ALPHA_AERO = 1.0, TLSAI_CRIT = 2.0;

inline double ipow4(double x) { double x2 = x * x; return x2 * x2; }
inline double ipow3(double x) { double x2 = x * x; return x2 * x; }

thread_local int t_err = 0, t_err_idx = 0;
void flag(int code, int idx) { if (!t_err) { t_err = code; t_err_idx = idx; } }

// QSatMod.F90:61-127 (Flatau et al. 1992 polynomials)
void qsat(double T, double p, double* qs, double* es, double* qsdT) {
    const double a0 = 6.11213476, a1 = 0.444007856, a2 = 0.143064234e-01, a3 = 0.264461437e-03,
                 a4 = 0.305903558e-05, a5 = 0.196237241e-07, a6 = 0.892344772e-10, a7 = -0.373208410e-12,
                 a8 = 0.209339997e-15;
    const double b0 = 0.444017302, b1 = 0.286064092e-01, b2 = 0.794683137e-03, b3 = 0.121211669e-04,
                 b4 = 0.103354611e-06, b5 = 0.404125005e-09, b6 = -0.788037859e-12, b7 = -0.114596802e-13,
                 b8 = 0.381294516e-16;
    const double c0 = 6.11123516, c1 = 0.503109514, c2 = 0.188369801e-01, c3 = 0.420547422e-03,
                 c4 = 0.614396778e-05, c5 = 0.602780717e-07, c6 = 0.387940929e-09, c7 = 0.149436277e-11,
                 c8 = 0.262655803e-14;
    const double d0 = 0.503277922, d1 = 0.377289173e-01, d2 = 0.126801703e-02, d3 = 0.249468427e-04,
                 d4 = 0.313703411e-06, d5 = 0.257180651e-08, d6 = 0.133268878e-10, d7 = 0.394116744e-13,
                 d8 = 0.498070196e-16;
    double td = std::min(100.0, std::max(-75.0, T - TFRZ));
    double esl;
    if (td >= 0.0)
        esl = a0 + td * (a1 + td * (a2 + td * (a3 + td * (a4 + td * (a5 + td * (a6 + td * (a7 + td * a8)))))));
    else
        esl = c0 + td * (c1 + td * (c2 + td * (c3 + td * (c4 + td * (c5 + td * (c6 + td * (c7 + td * c8)))))));
    esl = esl * 100.0;
    double vp = 1.0 / (p - 0.378 * esl);
    double vp1 = 0.622 * vp;
    *qs = esl * vp1;
    if (es) *es = esl;
    if (qsdT) {
        double esdT;
        if (td >= 0.0)
            esdT = b0 + td * (b1 + td * (b2 + td * (b3 + td * (b4 + td * (b5 + td * (b6 + td * (b7 + td * b8)))))));
        else
            esdT = d0 + td * (d1 + td * (d2 + td * (d3 + td * (d4 + td * (d5 + td * (d6 + td * (d7 + td * d8)))))));
        esdT = esdT * 100.0;
        double vp2 = vp1 * vp;
        *qsdT = esdT * vp2 * p;
    }
}

// quadraticMod.F90:17-74; returns 0 or CTSMG_E_DISCRIMINANT (roots then 0)
int quadratic(double a, double b, double c, double* r1, double* r2) {
    if (a == 0.0) { *r1 = *r2 = 0.0; return CTSMG_E_DISCRIMINANT; }
    double root = b * b - 4.0 * a * c;
    if (root < 0.0) {
        if (-root < 3.0 * 2.220446049250313e-16) root = 0.0;
        else { *r1 = *r2 = 0.0; return CTSMG_E_DISCRIMINANT; }
    }
    double q;
    if (b >= 0.0) q = -0.5 * (b + std::sqrt(root));
    else q = -0.5 * (b - std::sqrt(root));
    *r1 = q / a;
    if (q != 0.0) *r2 = c / q;
    else *r2 = 1.e36;
    return 0;
}

// FrictionVelocityMod.F90:1120-1155
double stab1(double zeta) {
    double chik2 = std::sqrt(1.0 - 16.0 * zeta);
    double chik = std::sqrt(chik2);
    return 2.0 * o_log((1.0 + chik) * 0.5) + o_log((1.0 + chik2) * 0.5) - 2.0 * o_atan(chik) + PI * 0.5;
}
double stab2(double zeta) {
    double chik2 = std::sqrt(1.0 - 16.0 * zeta);
    return 2.0 * o_log((1.0 + chik2) * 0.5);
}

// state of one photosynthesis evaluation (photosyns_inst components that
// ci_func writes: ac, aj, ap, ag, an; gs_mol is shared by both phases)
struct PsnState {
    double ac, aj, ap, ag, an, gs_mol;
};

struct PsnCtx {   // per patch-phase inputs of ci_func
    bool c3;
    double vcmax_z, cp, kc, ko, qe, tpu_z, kp_z, theta_cj, theta_ip, forc_pbot, medlynslope, medlynintercept;
    double bbb, mbb;
    int method;   // 1 = Medlyn, 0 = Ball-Berry
    double gb_mol, je, cair, oair, lmr_z, par_z, rh_can;
    int pidx;
};

// PhotosynthesisMod.F90:2564-2701
double ci_func(double ci, const PsnCtx& x, PsnState& s) {
    const double max_cs = 1.e-06;
    if (x.c3) {
        s.ac = x.vcmax_z * std::max(ci - x.cp, 0.0) / (ci + x.kc * (1.0 + x.oair / x.ko));
        s.aj = x.je * std::max(ci - x.cp, 0.0) / (4.0 * ci + 8.0 * x.cp);
        s.ap = 3.0 * x.tpu_z;
    } else {
        s.ac = x.vcmax_z;
        s.aj = x.qe * x.par_z * 4.6;
        s.ap = x.kp_z * std::max(ci, 0.0) / x.forc_pbot;
    }
    double r1, r2;
    if (quadratic(x.theta_cj, -(s.ac + s.aj), s.ac * s.aj, &r1, &r2)) flag(CTSMG_E_DISCRIMINANT, x.pidx);
    double ai = std::min(r1, r2);
    if (quadratic(x.theta_ip, -(ai + s.ap), ai * s.ap, &r1, &r2)) flag(CTSMG_E_DISCRIMINANT, x.pidx);
    s.ag = std::max(0.0, std::min(r1, r2));
    s.an = s.ag - x.lmr_z;
    if (s.an < 0.0) return 0.0;
    double cs = x.cair - 1.4 / x.gb_mol * s.an * x.forc_pbot;
    cs = std::max(cs, max_cs);
    if (x.method == 1) {
        double term = 1.6 * s.an / (cs / x.forc_pbot * 1.e06);
        double aquad = 1.0;
        double bquad = -(2.0 * (x.medlynintercept * 1.e-06 + term) +
                         (x.medlynslope * term) * (x.medlynslope * term) / (x.gb_mol * 1.e-06 * x.rh_can));
        double cquad = x.medlynintercept * x.medlynintercept * 1.e-12 +
                       (2.0 * x.medlynintercept * 1.e-06 + term * (1.0 - x.medlynslope * x.medlynslope / x.rh_can)) * term;
        if (quadratic(aquad, bquad, cquad, &r1, &r2)) flag(CTSMG_E_DISCRIMINANT, x.pidx);
        s.gs_mol = std::max(r1, r2) * 1.e06;
    } else {
        double aquad = cs;
        double bquad = cs * (x.gb_mol - x.bbb) - x.mbb * s.an * x.forc_pbot;
        double cquad = -x.gb_mol * (cs * x.bbb + x.mbb * s.an * x.forc_pbot * x.rh_can);
        if (quadratic(aquad, bquad, cquad, &r1, &r2)) flag(CTSMG_E_DISCRIMINANT, x.pidx);
        s.gs_mol = std::max(r1, r2);
    }
    return ci - x.cair + s.an * x.forc_pbot * (1.4 * s.gs_mol + 1.6 * x.gb_mol) / (x.gb_mol * s.gs_mol);
}

// PhotosynthesisMod.F90:2371-2485, for any evaluated function fn(x);
// *not_bracketed is the endrun condition of :2412-2415.
template <class F>
double brent_t(double x1, double x2, double f1, double f2, double tol, F&& fn, bool* not_bracketed) {
    const int itmax = 20;
    const double eps = 1.e-2;
    double a = x1, b = x2, fa = f1, fb = f2;
    if ((fa > 0.0 && fb > 0.0) || (fa < 0.0 && fb < 0.0)) {
        *not_bracketed = true;
        return b;
    }
    double c = b, fc = fb, d = 0.0, e = 0.0;
    int iter = 0;
    for (;;) {
        if (iter == itmax) break;
        iter = iter + 1;
        if ((fb > 0.0 && fc > 0.0) || (fb < 0.0 && fc < 0.0)) {
            c = a; fc = fa; d = b - a; e = d;
        }
        if (std::fabs(fc) < std::fabs(fb)) {
            a = b; b = c; c = a;
            fa = fb; fb = fc; fc = fa;
        }
        double tol1 = 2.0 * eps * std::fabs(b) + 0.5 * tol;
        double xm = 0.5 * (c - b);
        if (std::fabs(xm) <= tol1 || fb == 0.) return b;
        if (std::fabs(e) >= tol1 && std::fabs(fa) > std::fabs(fb)) {
            double s = fb / fa, p, q;
            if (a == c) {
                p = 2.0 * xm * s;
                q = 1.0 - s;
            } else {
                q = fa / fc;
                double r = fb / fc;
                p = s * (2.0 * xm * q * (q - r) - (b - a) * (r - 1.0));
                q = (q - 1.0) * (r - 1.0) * (s - 1.0);
            }
            if (p > 0.0) q = -q;
            p = std::fabs(p);
            if (2.0 * p < std::fmin(3.0 * xm * q - std::fabs(tol1 * q), std::fabs(e * q))) {
                e = d;
                d = p / q;
            } else {
                d = xm;
                e = d;
            }
        } else {
            d = xm;
            e = d;
        }
        a = b;
        fa = fb;
        if (std::fabs(d) > tol1) b = b + d;
        else b = b + std::copysign(std::fabs(tol1), xm);
        fb = fn(b);
        if (fb == 0.0) break;
    }
    return b;
}

// PhotosynthesisMod.F90:2251-2368; x0 in/out
template <class F>
void hybrid_t(double& x0, F&& fn, bool* not_bracketed) {
    const double eps = 1.e-2, eps1 = 1.e-4;
    const int itmax = 40;
    double f0 = fn(x0);
    if (f0 == 0.0) return;
    double minx = x0, minf = f0;
    double x1 = x0 * 0.99;
    double f1 = fn(x1);
    if (f1 == 0.0) { x0 = x1; return; }
    if (f1 < minf) { minx = x1; minf = f1; }
    int iter = 0;
    for (;;) {
        iter = iter + 1;
        double dx = -f1 * (x1 - x0) / (f1 - f0);
        double x = x1 + dx;
        double tol = std::fabs(x) * eps;
        if (std::fabs(dx) < tol) { x0 = x; break; }
        x0 = x1;
        f0 = f1;
        x1 = x;
        f1 = fn(x1);
        if (f1 < minf) { minx = x1; minf = f1; }
        if (std::fabs(f1) <= eps1) { x0 = x1; break; }
        if (f1 * f0 < 0.0) {
            x = brent_t(x0, x1, f0, f1, tol, fn, not_bracketed);
            x0 = x;
            break;
        }
        if (iter > itmax) {
            f1 = fn(minx);
            break;
        }
    }
}

void hybrid(double& x0, const PsnCtx& ctx, PsnState& st) {
    bool nb = false;
    hybrid_t(x0, [&](double x) { return ci_func(x, ctx, st); }, &nb);
    if (nb) flag(CTSMG_E_NOT_BRACKETED, ctx.pidx);
}

struct Params { ctsmg_canopy_params c; ctsmg_pftcon pft; int method; int itmax; };
Params g_par;
// optional per-patch Medlyn parameters (ensemble members), indexed by the
// 1-based global patch index minus 1
const double* g_mslope_p = nullptr;
const double* g_mint_p = nullptr;

double ft(double tl, double ha) { return o_exp(ha / (RGAS * 1.e-3 * (TFRZ + 25.0)) * (1.0 - (TFRZ + 25.0) / tl)); }
double fth(double tl, double hd, double se, double sf) { return sf / (1.0 + o_exp((-hd + se * tl) / (RGAS * 1.e-3 * tl))); }
double fth25(double hd, double se) { return 1.0 + o_exp((-hd + se * (TFRZ + 25.0)) / (RGAS * 1.e-3 * (TFRZ + 25.0))); }

struct PhaseOut { double rs, psn, lmr, ci, gs_mol_phase; };

// Photosynthesis (PhotosynthesisMod.F90:1243-2062) for one patch and phase,
// nlevcan = nrad = 1, satellite phenology, no LUNA / ozone.
PhaseOut photosynthesis(int pidx, int ivt, double t_veg, double t10, double tgcm, double forc_pbot,
                        double esat_tv, double eair, double oair, double cair, double rb, double btran,
                        double dayl_factor, double par_z, double lai_z, double vcmaxcint, PsnState& st,
                        double* vpd_can, double* rh_leaf) {
    const ctsmg_canopy_params& P = g_par.c;
    const ctsmg_pftcon& F = g_par.pft;
    const int method = g_par.method;
    const double medlyn_int = g_mint_p ? g_mint_p[pidx - 1] : F.medlynintercept[ivt];
    const double lmrc = fth25(P.lmrhd, P.lmrse);
    const bool c3 = (std::lround(F.c3psn[ivt]) == 1);
    const double qe = c3 ? 0.0 : 0.05;
    double bbb = 0.0, mbb = 0.0;
    if (method == 0) {
        const double bbbopt = c3 ? 10000.0 : 40000.0;
        bbb = std::max(bbbopt * btran, 1.0);
        mbb = F.mbbopt[ivt];
    }
    const double kc25 = P.kc25_coef * forc_pbot;
    const double ko25 = P.ko25_coef * forc_pbot;
    const double sco = 0.5 * 0.209 / P.cp25_yr2000;
    const double cp25 = 0.5 * oair / sco;
    const double kc = kc25 * ft(t_veg, P.kcha);
    const double ko = ko25 * ft(t_veg, P.koha);
    const double cp = cp25 * ft(t_veg, P.cpha);
    if (F.slatop[ivt] * F.leafcn[ivt] <= 0.0) flag(CTSMG_E_ARG, pidx);
    const double lnc = 1.0 / (F.slatop[ivt] * F.leafcn[ivt]);
    double vcmax25top = lnc * F.flnr[ivt] * P.fnr * P.act25 * dayl_factor;
    vcmax25top = vcmax25top * F.fnitr[ivt];
    const double t10c = std::min(std::max((t10 - TFRZ), 11.0), 35.0);
    const double jmax25top = ((2.59 - 0.035 * t10c) * vcmax25top) * P.jmax25top_sf;
    const double tpu25top = P.tpu25ratio * vcmax25top;
    const double kp25top = P.kp25ratio * vcmax25top;
    const double lmr25top = c3 ? vcmax25top * P.leaf_mr_vcm : vcmax25top * 0.025;
    const double nscaler = vcmaxcint;
    const double lmr25 = lmr25top * nscaler;
    double lmr_z;
    if (c3) {
        lmr_z = lmr25 * ft(t_veg, P.lmrha) * fth(t_veg, P.lmrhd, P.lmrse, lmrc);
    } else {
        lmr_z = lmr25 * o_pow(2.0, (t_veg - (TFRZ + 25.0)) / 10.0);
        lmr_z = lmr_z / (1.0 + o_exp(1.3 * (t_veg - (TFRZ + 55.0))));
    }
    double vcmax_z, jmax_z, tpu_z, kp_z;
    if (par_z <= 0.0) {
        vcmax_z = jmax_z = tpu_z = kp_z = 0.0;
    } else {
        const double vcmax25 = vcmax25top * nscaler, jmax25 = jmax25top * nscaler, tpu25 = tpu25top * nscaler;
        const double kp25 = kp25top * nscaler;
        const double vcmaxse = (668.39 - 1.07 * t10c) * P.vcmaxse_sf;
        const double jmaxse = (659.70 - 0.75 * t10c) * P.jmaxse_sf;
        const double tpuse = (668.39 - 1.07 * t10c) * P.tpuse_sf;
        const double vcmaxc = fth25(P.vcmaxhd, vcmaxse), jmaxc = fth25(P.jmaxhd, jmaxse), tpuc = fth25(P.tpuhd, tpuse);
        vcmax_z = vcmax25 * ft(t_veg, P.vcmaxha) * fth(t_veg, P.vcmaxhd, vcmaxse, vcmaxc);
        jmax_z = jmax25 * ft(t_veg, P.jmaxha) * fth(t_veg, P.jmaxhd, jmaxse, jmaxc);
        tpu_z = tpu25 * ft(t_veg, P.tpuha) * fth(t_veg, P.tpuhd, tpuse, tpuc);
        if (!c3) {
            vcmax_z = vcmax25 * o_pow(2.0, (t_veg - (TFRZ + 25.0)) / 10.0);
            vcmax_z = vcmax_z / (1.0 + o_exp(0.2 * ((TFRZ + 15.0) - t_veg)));
            vcmax_z = vcmax_z / (1.0 + o_exp(0.3 * (t_veg - (TFRZ + 40.0))));
        }
        kp_z = kp25 * o_pow(2.0, (t_veg - (TFRZ + 25.0)) / 10.0);
    }
    vcmax_z = vcmax_z * btran;
    lmr_z = lmr_z * btran;
    if (P.light_inhibit && par_z > 0.0) lmr_z = lmr_z * 0.67;

    const double rsmax0 = 2.e4;
    const double cf = forc_pbot / (RGAS * 1.e-3 * tgcm) * 1.e06;
    const double gb = 1.0 / rb;
    const double gb_mol = gb * cf;
    PhaseOut out;
    double rs_z, psn_z, ci_z;
    if (par_z <= 0.0) {
        st.ac = st.aj = st.ap = st.ag = 0.0;
        st.an = st.ag - lmr_z;
        psn_z = 0.0;
        if (method == 0) rs_z = std::min(rsmax0, 1.0 / bbb * cf);
        else rs_z = std::min(rsmax0, 1.0 / medlyn_int * cf);
        ci_z = 0.0;
        *rh_leaf = 0.0;
        out.gs_mol_phase = cf / rs_z;
    } else {
        const double ceair = std::min(eair, esat_tv);
        double rh_can;
        if (method == 0) {
            rh_can = ceair / esat_tv;
        } else {
            rh_can = std::max((esat_tv - ceair), 50.0) * 0.001;
            *vpd_can = rh_can;
        }
        const double qabs = 0.5 * (1.0 - P.fnps) * par_z * 4.6;
        double r1, r2;
        if (quadratic(P.theta_psii, -(qabs + jmax_z), qabs * jmax_z, &r1, &r2)) flag(CTSMG_E_DISCRIMINANT, pidx);
        const double je = std::min(r1, r2);
        ci_z = c3 ? 0.7 * cair : 0.4 * cair;
        PsnCtx ctx{c3, vcmax_z, cp, kc, ko, qe, tpu_z, kp_z, F.theta_cj[ivt], P.theta_ip, forc_pbot,
                   g_mslope_p ? g_mslope_p[pidx - 1] : F.medlynslope[ivt], medlyn_int, bbb, mbb, method, gb_mol, je,
                   cair, oair, lmr_z, par_z, rh_can, pidx};
        double ciold = ci_z;
        hybrid(ciold, ctx, st);
        if (st.an < 0.0) st.gs_mol = (method == 0) ? bbb : medlyn_int;
        out.gs_mol_phase = st.gs_mol;
        double cs = cair - 1.4 / gb_mol * st.an * forc_pbot;
        cs = std::max(cs, 1.e-06);
        ci_z = cair - st.an * forc_pbot * (1.4 * st.gs_mol + 1.6 * gb_mol) / (gb_mol * st.gs_mol);
        ci_z = std::max(ci_z, 1.e-06);
        const double gs = st.gs_mol / cf;
        rs_z = std::min(1.0 / gs, rsmax0);
        rs_z = rs_z / 1.0;
        psn_z = st.ag;
        psn_z = psn_z * 1.0;
        if (st.gs_mol < 0.0) flag(CTSMG_E_ARG, pidx);
        if (method == 0) {
            double hs = (gb_mol * ceair + st.gs_mol * esat_tv) / ((gb_mol + st.gs_mol) * esat_tv);
            *rh_leaf = hs;
        }
    }
    const double psncan = psn_z * lai_z, lmrcan = lmr_z * lai_z, gscan = lai_z / (rb + rs_z), laican = lai_z;
    if (laican > 0.0) {
        out.psn = psncan / laican;
        out.lmr = lmrcan / laican;
        out.rs = laican / gscan - rb;
    } else {
        out.psn = 0.0; out.lmr = 0.0; out.rs = 0.0;
    }
    out.ci = ci_z;
    return out;
}

// FrictionVelocityMod.F90:754-1117 for one patch
struct FVOut { double ustar, temp1, temp2, temp12m, temp22m, u10_clm, va, vds, u10, fv; };
void friction_velocity(double displa, double z0m, double z0h, double z0q, double obu, int iter, double ur,
                       double um, double hgt_u, double hgt_t, double hgt_q, double& fm, FVOut& o) {
    const double zetam = 1.574, zetat = 0.465;
    double zldis = hgt_u - displa;
    double zeta = zldis / obu;
    double ustar;
    if (zeta < -zetam) {
        ustar = VKC * um / (o_log(-zetam * obu / z0m) - stab1(-zetam) + stab1(z0m / obu) +
                            1.14 * (o_pow(-zeta, 0.333) - o_pow(zetam, 0.333)));
    } else if (zeta < 0.0) {
        ustar = VKC * um / (o_log(zldis / z0m) - stab1(zeta) + stab1(z0m / obu));
    } else if (zeta <= 1.0) {
        ustar = VKC * um / (o_log(zldis / z0m) + 5.0 * zeta - 5.0 * z0m / obu);
    } else {
        ustar = VKC * um / (o_log(obu / z0m) + 5.0 - 5.0 * z0m / obu + (5.0 * o_log(zeta) + zeta - 1.0));
    }
    o.ustar = ustar;
    if (zeta < 0.0) o.vds = 2.e-3 * ustar * (1.0 + o_pow(300.0 / (-obu), 0.666));
    else o.vds = 2.e-3 * ustar;
    if (zldis - z0m <= 10.0) {
        o.u10_clm = um;
    } else {
        const double z10 = 10.0 + z0m;
        if (zeta < -zetam)
            o.u10_clm = um - (ustar / VKC * (o_log(-zetam * obu / z10) - stab1(-zetam) + stab1(z10 / obu) +
                                              1.14 * (o_pow(-zeta, 0.333) - o_pow(zetam, 0.333))));
        else if (zeta < 0.0)
            o.u10_clm = um - (ustar / VKC * (o_log(zldis / z10) - stab1(zeta) + stab1(z10 / obu)));
        else if (zeta <= 1.0)
            o.u10_clm = um - (ustar / VKC * (o_log(zldis / z10) + 5.0 * zeta - 5.0 * z10 / obu));
        else
            o.u10_clm = um - (ustar / VKC * (o_log(obu / z10) + 5.0 - 5.0 * z10 / obu + (5.0 * o_log(zeta) + zeta - 1.0)));
    }
    o.va = um;
    auto tprof = [&](double zl, double z0) {
        double zt = zl / obu;
        if (zt < -zetat)
            return VKC / (o_log(-zetat * obu / z0) - stab2(-zetat) + stab2(z0 / obu) +
                          0.8 * (o_pow(zetat, -0.333) - o_pow(-zt, -0.333)));
        else if (zt < 0.0)
            return VKC / (o_log(zl / z0) - stab2(zt) + stab2(z0 / obu));
        else if (zt <= 1.0)
            return VKC / (o_log(zl / z0) + 5.0 * zt - 5.0 * z0 / obu);
        else
            return VKC / (o_log(obu / z0) + 5.0 - 5.0 * z0 / obu + (5.0 * o_log(zt) + zt - 1.0));
    };
    o.temp1 = tprof(hgt_t - displa, z0h);
    if (hgt_q == hgt_t && z0q == z0h) o.temp2 = o.temp1;
    else o.temp2 = tprof(hgt_q - displa, z0q);
    o.temp12m = tprof(2.0 + z0h, z0h);
    if (z0q == z0h) o.temp22m = o.temp12m;
    else o.temp22m = tprof(2.0 + z0q, z0q);
    zldis = hgt_u - displa;
    zeta = zldis / obu;
    double fmnew;
    if (std::min(zeta, 1.0) < 0.0) {
        double tmp1 = o_pow(1.0 - 16.0 * std::min(zeta, 1.0), 0.25);
        double tmp2 = o_log((1.0 + tmp1 * tmp1) / 2.0);
        double tmp3 = o_log((1.0 + tmp1) / 2.0);
        fmnew = 2.0 * tmp3 + tmp2 - 2.0 * o_atan(tmp1) + 1.5707963;
    } else {
        fmnew = -5.0 * std::min(zeta, 1.0);
    }
    if (iter == 1) fm = fmnew;
    else fm = 0.5 * (fm + fmnew);
    double zeta10 = std::min(10.0 / obu, 1.0);
    if (zeta == 0.0) zeta10 = 0.0;
    double fm10;
    if (zeta10 < 0.0) {
        double tmp1 = o_pow(1.0 - 16.0 * zeta10, 0.25);
        double tmp2 = o_log((1.0 + tmp1 * tmp1) / 2.0);
        double tmp3 = o_log((1.0 + tmp1) / 2.0);
        fm10 = 2.0 * tmp3 + tmp2 - 2.0 * o_atan(tmp1) + 1.5707963;
    } else {
        fm10 = -5.0 * zeta10;
    }
    double tmp4 = o_log(std::max(1.0, hgt_u / 10.0));
    o.u10 = ur - ustar / VKC * (tmp4 - fm + fm10);
    o.fv = ustar;
}

// CanopyFluxes (CanopyFluxesMod.F90:642-1655) for one patch
void canopy_patch(int p, const ctsmg_bounds* b, const ctsmg_canopy_io* io, double dtime) {
    const ctsmg_canopy_params& P = g_par.c;
    const int pg = p + b->begp;
    const int c = io->patch_column[p] - b->begc;
    const int g = io->patch_gridcell[p] - io->begg;
    const int ivt = io->itype[p];
    const int ldc = io->ldc;
    auto TS = [&](int j) { return io->t_soisno[c + (size_t)(j + CTSMG_NLEVSNO - 1) * ldc]; };
    const double delmax = 1.0, dlemin = 0.1, dtmin = 0.01, zii = 1000.0, beta = 1.0, btran0 = 0.0;
    const int itmin = 2;

    const double elai = io->elai[p], esai = io->esai[p], emv = io->emv[p], emg = io->emg[c];
    const double forc_pbot = io->forc_pbot[c], forc_q = io->forc_q[c], forc_th = io->forc_th[c];
    const double forc_rho = io->forc_rho[c], thv = io->thv[c], t_grnd = io->t_grnd[c], qg = io->qg[c];
    const double thm = io->thm[p], btran = io->btran[p], htvp = io->htvp[c];
    const double fv = (double)io->frac_veg_nosno[p];

    double del = 0.0, efeb = 0.0, wtlq0 = 0.0, wtalq = 0.0, wtgq = 0.0, wtaq0 = 0.0, obuold = 0.0;
    const double sa_leaf = (elai + esai), frac_rad_abs_by_stem = 0.0, sa_stem = 0.0, sa_internal = 0.0;
    const double cp_leaf = 0.0, rstem = 0.0;
    (void)sa_stem;
    const double dayl_factor = std::min(1.0, std::max(0.01, (io->dayl[g] * io->dayl[g]) / (io->max_dayl[g] * io->max_dayl[g])));
    io->rb1[p] = 0.0;
    // ZengWang2007 roughness (:905-911)
    double lt = std::min(elai + esai, TLSAI_CRIT);
    double egvf = (1.0 - ALPHA_AERO * o_exp(-lt)) / (1.0 - ALPHA_AERO * o_exp(-TLSAI_CRIT));
    double displa = egvf * io->displa[p];
    double z0mv = o_exp(egvf * o_log(io->z0mv[p]) + (1.0 - egvf) * o_log(io->z0mg[c]));
    io->displa[p] = displa;
    io->z0mv[p] = z0mv;
    const double z0hv = z0mv, z0qv = z0mv;
    io->z0hv[p] = z0hv;
    io->z0qv[p] = z0qv;
    const double hgt_u = io->forc_hgt_u[g] + z0mv + displa;
    const double hgt_t = io->forc_hgt_t[g] + z0hv + displa;
    const double hgt_q = io->forc_hgt_q[g] + z0qv + displa;
    io->forc_hgt_u_patch[p] = hgt_u;
    io->forc_hgt_t_patch[p] = hgt_t;
    io->forc_hgt_q_patch[p] = hgt_q;

    const double air = emv * (1.0 + (1.0 - emv) * (1.0 - emg)) * io->forc_lwrad[c];
    const double bir = -(2.0 - emv * (1.0 - emg)) * emv * SB;
    const double cir = emv * emg * SB;
    double t_veg = io->t_veg[p];
    double qsatl, el, qsatldT;
    qsat(t_veg, forc_pbot, &qsatl, &el, &qsatldT);
    const double co2 = io->forc_pco2[g], o2 = io->forc_po2[g];
    int nmozsgn = 0;
    double taf = (t_grnd + thm) / 2.0;
    double qaf = (forc_q + qg) / 2.0;
    const double ur = std::max(P.wind_min, std::sqrt(io->forc_u[g] * io->forc_u[g] + io->forc_v[g] * io->forc_v[g]));
    double dth = thm - taf;
    double dqh = forc_q - qaf;
    double delq = qg - qaf;
    double dthv = dth * (1.0 + 0.61 * forc_q) + 0.61 * forc_th * dqh;
    const double zldis = hgt_u - displa;
    if (zldis < 0.0) flag(CTSMG_E_FORCING_HEIGHT, pg);
    // MoninObukIni (FrictionVelocityMod.F90:1158-1209)
    double um, obu;
    {
        const double wc = 0.5;
        if (dthv >= 0.0) um = std::max(ur, 0.1);
        else um = std::sqrt(ur * ur + wc * wc);
        double rib = GRAV * zldis * dthv / (thv * um * um);
        double zeta;
        if (rib >= 0.0) {
            zeta = rib * o_log(zldis / z0mv) / (1.0 - 5.0 * std::min(rib, 0.19));
            zeta = std::min(P.zetamaxstable, std::max(zeta, 0.01));
        } else {
            zeta = rib * o_log(zldis / z0mv);
            zeta = std::max(-100.0, std::min(zeta, -0.01));
        }
        obu = zldis / zeta;
    }
    int num_iter = 0;
    const double tl_ini = t_veg;
    double liqcan = io->liqcan[p], snocan = io->snocan[p];
    const double fwet = io->fwet[p], fdry = io->fdry[p], laisun = io->laisun[p], laisha = io->laisha[p];
    const double snl = io->snl[c];
    const double frac_sno = io->frac_sno_eff[c], frac_h2osfc = io->frac_h2osfc[c];
    double fm = 0.0;
    double rb = 0.0, ram1 = 0.0, rah_a = 0.0, raw_a = 0.0, rah_b = 0.0, raw_b = 0.0, uaf = 0.0;
    double temp1 = 0, temp2 = 0, temp12m = 0, temp22m = 0, ustar = 0;
    double wtl0 = 0, wta0 = 0, wtg = 0, wtal = 0, wtga = 0, wtstem0 = 0;
    double efe = 0.0, tlbef = t_veg, dt_veg = 0.0, err = 0.0, eflx_sh_veg = 0.0, qflx_evap_veg = 0.0;
    double qflx_tran_veg = 0.0, lw_leaf = 0.0, zeta_out = 0.0;
    PsnState st{0, 0, 0, 0, 0, 0};
    PhaseOut sun{}, sha{};
    double vpd_can = 0.0, rh_leaf = 0.0;
    FVOut fo{};
    int itlef = 0;
    while (itlef <= g_par.itmax) {
        friction_velocity(displa, z0mv, z0hv, z0qv, obu, itlef + 1, ur, um, hgt_u, hgt_t, hgt_q, fm, fo);
        ustar = fo.ustar; temp1 = fo.temp1; temp2 = fo.temp2; temp12m = fo.temp12m; temp22m = fo.temp22m;
        tlbef = t_veg;
        const double del2 = del;
        ram1 = 1.0 / (ustar * ustar / um);
        rah_a = 1.0 / (temp1 * ustar);
        raw_a = 1.0 / (temp2 * ustar);
        uaf = um * std::sqrt(1.0 / (ram1 * um));
        const double dleaf = g_par.pft.dleaf[ivt];
        const double cf = P.cv / (std::sqrt(uaf) * std::sqrt(dleaf));
        rb = 1.0 / (cf * uaf);
        io->rb1[p] = rb;
        const double w = o_exp(-(elai + esai));
        const double csoilb = VKC / (P.a_coef * o_pow(io->z0mg[c] * uaf / NU_PARAM, P.a_exp));
        const double csoilcn = csoilb * w + P.csoilc * (1.0 - w);
        rah_b = 1.0 / (csoilcn * uaf);
        raw_b = rah_b;
        const double svpts = el;
        const double eah = forc_pbot * qaf / 0.622;
        io->rhaf[p] = eah / svpts;
        io->vpd[p] = std::max((svpts - eah), 50.0) * 0.001;

        sun = photosynthesis(pg, ivt, t_veg, io->t_a10[p], thm, forc_pbot, svpts, eah, o2, co2, rb, btran, dayl_factor,
                             io->parsun_z[p], laisun, io->vcmaxcintsun[p], st, &vpd_can, &rh_leaf);
        sha = photosynthesis(pg, ivt, t_veg, io->t_a10[p], thm, forc_pbot, svpts, eah, o2, co2, rb, btran, dayl_factor,
                             io->parsha_z[p], laisha, io->vcmaxcintsha[p], st, &vpd_can, &rh_leaf);

        const double wta = 1.0 / rah_a;
        const double wtl = sa_leaf / rb;
        wtg = 1.0 / rah_b;
        const double wtstem = 0.0 / (rstem + rb);
        const double wtshi = 1.0 / (wta + wtl + wtstem + wtg);
        wtl0 = wtl * wtshi;
        const double wtg0 = wtg * wtshi;
        wta0 = wta * wtshi;
        wtstem0 = wtstem * wtshi;
        wtga = wta0 + wtg0 + wtstem0;
        wtal = wta0 + wtl0 + wtstem0;
        const double lw_stem = 0.0;
        lw_leaf = 0.0;
        double rppdry;
        if (fdry > 0.0) rppdry = fdry * rb * (laisun / (rb + sun.rs) + laisha / (rb + sha.rs)) / elai;
        else rppdry = 0.0;
        double efpot = forc_rho * ((elai + esai) / rb) * (qsatl - qaf);
        const double h2ocan = liqcan + snocan;
        double rpp;
        if (efpot > 0.0) {
            if (btran > btran0) {
                qflx_tran_veg = efpot * rppdry;
                rpp = rppdry + fwet;
            } else {
                rpp = fwet;
                qflx_tran_veg = 0.0;
            }
            rpp = std::min(rpp, (qflx_tran_veg + h2ocan / dtime) / efpot);
        } else {
            rpp = 1.0;
            qflx_tran_veg = 0.0;
        }
        const double wtaq = fv / raw_a;
        const double wtlq = fv * (elai + esai) / rb * rpp;
        const double snow_depth_c = P.z_dl;
        const double fsno_dl = io->snow_depth[c] / snow_depth_c;
        const double elai_dl = P.lai_dl * (1.0 - std::min(fsno_dl, 1.0));
        const double rdl = (1.0 - o_exp(-elai_dl)) / (0.004 * uaf);
        if (delq < 0.0) wtgq = fv / (raw_b + rdl);
        else wtgq = fv / (raw_b + io->soilresis[c]);
        const double wtsqi = 1.0 / (wtaq + wtlq + wtgq);
        const double wtgq0 = wtgq * wtsqi;
        wtlq0 = wtlq * wtsqi;
        wtaq0 = wtaq * wtsqi;
        const double wtgaq = wtaq0 + wtgq0;
        wtalq = wtaq0 + wtlq0;
        const double dc1 = forc_rho * CPAIR * wtl;
        const double dc2 = HVAP * forc_rho * wtlq;
        const double efsh = dc1 * (wtga * t_veg - wtg0 * t_grnd - wta0 * thm - wtstem0 * 0.0);
        efe = dc2 * (wtgaq * qsatl - wtgq0 * qg - wtaq0 * forc_q);
        double erre = 0.0;
        if (efe * efeb < 0.0) {
            const double efeold = efe;
            efe = 0.1 * efeold;
            erre = efe - efeold;
        }
        const double lw_grnd = (frac_sno * ipow4(TS((int)snl + 1)) + (1.0 - frac_sno - frac_h2osfc) * ipow4(TS(1)) +
                                frac_h2osfc * ipow4(io->t_h2osfc[c]));
        dt_veg = ((1.0 - frac_rad_abs_by_stem) * (io->sabv[p] + air + bir * ipow4(t_veg) + cir * lw_grnd) - efsh - efe -
                  lw_leaf + lw_stem - (cp_leaf / dtime) * (t_veg - tl_ini)) /
                 ((1.0 - frac_rad_abs_by_stem) * (-4.0 * bir * ipow3(t_veg)) + 4.0 * sa_internal * emv * SB * ipow3(t_veg) +
                  dc1 * wtga + dc2 * wtgaq * qsatldT + cp_leaf / dtime);
        t_veg = tlbef + dt_veg;
        const double dels = dt_veg;
        del = std::fabs(dels);
        err = 0.0;
        if (del > delmax) {
            dt_veg = delmax * dels / del;
            t_veg = tlbef + dt_veg;
            err = (1.0 - frac_rad_abs_by_stem) * (io->sabv[p] + air + bir * ipow3(tlbef) * (tlbef + 4.0 * dt_veg) + cir * lw_grnd) -
                  sa_internal * emv * SB * ipow3(tlbef) * (tlbef + 4.0 * dt_veg) + lw_stem -
                  (efsh + dc1 * wtga * dt_veg) - (efe + dc2 * wtgaq * qsatldT * dt_veg) - (cp_leaf / dtime) * (t_veg - tl_ini);
        }
        efpot = forc_rho * ((elai + esai) / rb) * (wtgaq * (qsatl + qsatldT * dt_veg) - wtgq0 * qg - wtaq0 * forc_q);
        qflx_evap_veg = rpp * efpot;
        double ecidif = 0.0;
        if (efpot > 0.0 && btran > btran0) qflx_tran_veg = efpot * rppdry;
        else qflx_tran_veg = 0.0;
        ecidif = std::max(0.0, qflx_evap_veg - qflx_tran_veg - h2ocan / dtime);
        qflx_evap_veg = std::min(qflx_evap_veg, qflx_tran_veg + h2ocan / dtime);
        eflx_sh_veg = efsh + dc1 * wtga * dt_veg + err + erre + HVAP * ecidif;
        lw_leaf = sa_internal * emv * SB * ipow3(tlbef) * (tlbef + 4.0 * dt_veg);
        qsat(t_veg, forc_pbot, &qsatl, &el, &qsatldT);
        taf = wtg0 * t_grnd + wta0 * thm + wtl0 * t_veg + wtstem0 * 0.0;
        qaf = wtlq0 * qsatl + wtgq0 * qg + forc_q * wtaq0;
        dth = thm - taf;
        dqh = forc_q - qaf;
        delq = wtalq * qg - wtlq0 * qsatl - wtaq0 * forc_q;
        const double tstar = temp1 * dth;
        const double qstar = temp2 * dqh;
        const double thvstar = tstar * (1.0 + 0.61 * forc_q) + 0.61 * forc_th * qstar;
        double zeta = zldis * VKC * GRAV * thvstar / ((ustar * ustar) * thv);
        if (zeta >= 0.0) {
            zeta = std::min(P.zetamaxstable, std::max(zeta, 0.01));
            um = std::max(ur, 0.1);
        } else {
            zeta = std::max(-100.0, std::min(zeta, -0.01));
            double wc;
            if (ustar * thvstar > 0.0) wc = 0.0;
            else wc = beta * o_pow(-GRAV * ustar * thvstar * zii / thv, 0.333);
            um = std::sqrt(ur * ur + wc * wc);
        }
        zeta_out = zeta;
        obu = zldis / zeta;
        if (obuold * obu < 0.0) nmozsgn = nmozsgn + 1;
        if (nmozsgn >= 4) obu = zldis / (-0.01);
        obuold = obu;
        itlef = itlef + 1;
        if (itlef > itmin) {
            const double dele = std::fabs(efe - efeb);
            efeb = efe;
            const double det = std::max(del, del2);
            num_iter = itlef;
            if (det < dtmin && dele < dlemin) break;
        }
    }

    // post-iteration (:1461-1655)
    const double lw_grnd = (frac_sno * ipow4(TS((int)snl + 1)) + (1.0 - frac_sno - frac_h2osfc) * ipow4(TS(1)) +
                            frac_h2osfc * ipow4(io->t_h2osfc[c]));
    err = (1.0 - frac_rad_abs_by_stem) * (io->sabv[p] + air + bir * ipow3(tlbef) * (tlbef + 4.0 * dt_veg) + cir * lw_grnd) -
          lw_leaf + 0.0 - eflx_sh_veg - HVAP * qflx_evap_veg - ((t_veg - tl_ini) * cp_leaf / dtime);
    const double dt_stem = 0.0;
    const double delt = wtal * t_grnd - wtl0 * t_veg - wta0 * thm - wtstem0 * 0.0;
    io->taux[p] = -forc_rho * io->forc_u[g] / ram1;
    io->tauy[p] = -forc_rho * io->forc_v[g] / ram1;
    io->eflx_sh_grnd[p] = CPAIR * forc_rho * wtg * delt;
    const double delt_snow = wtal * TS((int)snl + 1) - wtl0 * t_veg - wta0 * thm - wtstem0 * 0.0;
    const double delt_soil = wtal * TS(1) - wtl0 * t_veg - wta0 * thm - wtstem0 * 0.0;
    const double delt_h2osfc = wtal * io->t_h2osfc[c] - wtl0 * t_veg - wta0 * thm - wtstem0 * 0.0;
    io->eflx_sh_snow[p] = CPAIR * forc_rho * wtg * delt_snow;
    io->eflx_sh_soil[p] = CPAIR * forc_rho * wtg * delt_soil;
    io->eflx_sh_h2osfc[p] = CPAIR * forc_rho * wtg * delt_h2osfc;
    io->qflx_evap_soi[p] = forc_rho * wtgq * delq;
    const double delq_snow = wtalq * io->qg_snow[c] - wtlq0 * qsatl - wtaq0 * forc_q;
    io->qflx_ev_snow[p] = forc_rho * wtgq * delq_snow;
    const double delq_soil = wtalq * io->qg_soil[c] - wtlq0 * qsatl - wtaq0 * forc_q;
    io->qflx_ev_soil[p] = forc_rho * wtgq * delq_soil;
    const double delq_h2osfc = wtalq * io->qg_h2osfc[c] - wtlq0 * qsatl - wtaq0 * forc_q;
    io->qflx_ev_h2osfc[p] = forc_rho * wtgq * delq_h2osfc;
    const double t_ref2m = thm + temp1 * dth * (1.0 / temp12m - 1.0 / temp1);
    const double q_ref2m = forc_q + temp2 * dqh * (1.0 / temp22m - 1.0 / temp2);
    double qsat_ref2m, e_ref2m;
    qsat(t_ref2m, forc_pbot, &qsat_ref2m, &e_ref2m, nullptr);
    const double rh_ref2m = std::min(100.0, q_ref2m / qsat_ref2m * 100.0);
    io->t_ref2m[p] = t_ref2m;
    io->q_ref2m[p] = q_ref2m;
    io->rh_ref2m[p] = rh_ref2m;
    io->vpd_ref2m[p] = e_ref2m * (1.0 - rh_ref2m / 100.0);
    const double ts_ini = 0.0;
    io->dlrad[p] = (1.0 - emv) * emg * io->forc_lwrad[c] +
                   emv * emg * SB * ipow3(tlbef) * (tlbef + 4.0 * dt_veg) * (1.0 - frac_rad_abs_by_stem) +
                   emv * emg * SB * ipow3(ts_ini) * (ts_ini + 4.0 * dt_stem) * frac_rad_abs_by_stem;
    io->ulrad[p] = ((1.0 - emg) * (1.0 - emv) * (1.0 - emv) * io->forc_lwrad[c] +
                    emv * (1.0 + (1.0 - emg) * (1.0 - emv)) * SB * ipow3(tlbef) * (tlbef + 4.0 * dt_veg) * (1.0 - frac_rad_abs_by_stem) +
                    emv * (1.0 + (1.0 - emg) * (1.0 - emv)) * SB * ipow3(ts_ini) * (ts_ini + 4.0 * dt_stem) * frac_rad_abs_by_stem +
                    emg * (1.0 - emv) * SB * lw_grnd);
    io->t_skin[p] = emv * t_veg + (1.0 - emv) * std::sqrt(std::sqrt(lw_grnd));
    const double cgrnds = io->cgrnds[p] + CPAIR * forc_rho * wtg * wtal;
    const double cgrndl = io->cgrndl[p] + forc_rho * wtgq * wtalq * io->dqgdT[c];
    io->cgrnds[p] = cgrnds;
    io->cgrndl[p] = cgrndl;
    io->cgrnd[p] = cgrnds + cgrndl * htvp;
    const double snocan_baseline = snocan;
    if (t_veg > TFRZ) {
        if ((qflx_evap_veg - qflx_tran_veg) * dtime > liqcan)
            snocan = std::max(0.0, snocan + liqcan + (qflx_tran_veg - qflx_evap_veg) * dtime);
        liqcan = std::max(0.0, liqcan + (qflx_tran_veg - qflx_evap_veg) * dtime);
    } else if (t_veg <= TFRZ) {
        if ((qflx_evap_veg - qflx_tran_veg) * dtime > snocan)
            liqcan = liqcan + snocan + (qflx_tran_veg - qflx_evap_veg) * dtime;
        snocan = std::max(0.0, snocan + (qflx_tran_veg - qflx_evap_veg) * dtime);
    }
    if (std::fabs(snocan) < 1.e-10 * std::fabs(snocan_baseline)) snocan = 0.0;   // truncate_small_values
    io->liqcan[p] = liqcan;
    io->snocan[p] = snocan;
    io->t_veg[p] = t_veg;
    io->taf[p] = taf;
    io->qaf[p] = qaf;
    io->ustar[p] = ustar;
    io->um[p] = um;
    io->obu[p] = obu;
    io->zeta[p] = zeta_out;
    io->ram1[p] = ram1;
    io->rah1[p] = rah_a;
    io->raw1[p] = raw_a;
    io->rah2[p] = rah_b;
    io->raw2[p] = raw_b;
    io->uaf[p] = uaf;
    io->eflx_sh_veg[p] = eflx_sh_veg;
    io->qflx_evap_veg[p] = qflx_evap_veg;
    io->qflx_tran_veg[p] = qflx_tran_veg;
    io->err_canopy[p] = err;
    io->num_iter[p] = num_iter;
    io->rssun[p] = sun.rs; io->rssha[p] = sha.rs;
    io->psnsun[p] = sun.psn; io->psnsha[p] = sha.psn;
    io->lmrsun[p] = sun.lmr; io->lmrsha[p] = sha.lmr;
    io->cisun[p] = sun.ci; io->cisha[p] = sha.ci;
    io->gs_mol_sun[p] = sun.gs_mol_phase; io->gs_mol_sha[p] = sha.gs_mol_phase;
    io->rh_leaf[p] = rh_leaf;
    io->vpd_can[p] = vpd_can;
    io->u10_clm[p] = fo.u10_clm; io->u10[p] = fo.u10; io->fv[p] = fo.fv; io->vds[p] = fo.vds;
    io->fm[p] = fm;
}

} // namespace

extern "C" void oracle_set_canopy_params(const ctsmg_canopy_params* p, const ctsmg_pftcon* pft, int method, int itmax) {
    g_par.c = *p;
    g_par.pft = *pft;
    g_par.method = method;
    g_par.itmax = itmax;
}

extern "C" void oracle_set_patch_medlyn(const double* slope, const double* intercept) {
    g_mslope_p = slope;
    g_mint_p = intercept;
}

// The points hybrid evaluates for one of the synthetic functions of
// rootfind_testfns.h (test support: pins the device root finder's control flow).
extern "C" int oracle_rootfind_trace(int k, const double* prm, double x0, double* xs, int cap, int* not_bracketed) {
    int n = 0;
    bool nb = false;
    hybrid_t(x0, [&](double x) { if (n < cap) xs[n] = x; ++n; return rf_testfn(k, prm, x); }, &nb);
    *not_bracketed = nb ? 1 : 0;
    return n;
}

extern "C" int oracle_quadratic(double a, double b, double c, double* r1, double* r2) {
    return quadratic(a, b, c, r1, r2);
}

extern "C" void oracle_qsat(double T, double p, double* qs, double* es, double* qsdT) { qsat(T, p, qs, es, qsdT); }

extern "C" int oracle_canopyfluxes(const ctsmg_bounds* b, int num_exposedvegp, const int32_t* filter_exposedvegp,
                                   const ctsmg_canopy_io* io, double dtime, int* err_index) {
    int code = 0, idx = 0;
#pragma omp parallel for schedule(dynamic, 64)
    for (int f = 0; f < num_exposedvegp; ++f) {
        t_err = 0;
        canopy_patch(filter_exposedvegp[f] - b->begp, b, io, dtime);
        if (t_err) {
#pragma omp critical
            { if (!code) { code = t_err; idx = t_err_idx; } }
        }
    }
    if (err_index) *err_index = idx;
    return code;
}

// CanopyFluxesMod.F90:709, 833-895 -> SoilMoistStressMod.F90:70-114 (effective
// porosity), 171-217 (volumetric liquid, jtop = 1), 312-435 (default stress,
// perchroot off) with the Clapp-Hornberger suction.
extern "C" int oracle_root_moist_stress(const ctsmg_bounds* b, int nump, const int32_t* filtp,
                                        const ctsmg_rootmoist_io* io) {
    const double TFRZ_ = 273.15, DENICE_ = 917.0, DENH2O_ = 1000.0;
    const int NLEVSNO_ = 12, NLEVGRND_ = 25, LS_ = -NLEVSNO_ + 1;
    const int ldc = io->ldc, ldp = io->ldp;
    std::vector<int> cols;
    for (int f = 0; f < nump; ++f) cols.push_back(io->patch_column[filtp[f] - b->begp] - b->begc);
    for (int j = 1; j <= NLEVGRND_; ++j)
        for (int c : cols) {
            const size_t ss = c + (size_t)(j - LS_) * ldc, g = c + (size_t)(j - 1) * ldc;
            const double vol_ice = std::min(io->watsat[g], io->h2osoi_ice[ss] / (DENICE_ * io->dz[ss]));
            io->eff_porosity[g] = io->watsat[g] - vol_ice;
        }
    for (int j = 1; j <= NLEVGRND_; ++j)
        for (int c : cols) {
            const size_t ss = c + (size_t)(j - LS_) * ldc, g = c + (size_t)(j - 1) * ldc;
            io->h2osoi_liqvol[g] = std::min(io->eff_porosity[g], io->h2osoi_liq[ss] / (io->dz[ss] * DENH2O_));
        }
    for (int f = 0; f < nump; ++f) io->btran[filtp[f] - b->begp] = 0.0;
    for (int j = 1; j <= NLEVGRND_; ++j)
        for (int f = 0; f < nump; ++f) {
            const int p = filtp[f] - b->begp, c = io->patch_column[p] - b->begc, it = io->itype[p];
            const size_t ss = c + (size_t)(j - LS_) * ldc, g = c + (size_t)(j - 1) * ldc, pg = p + (size_t)(j - 1) * ldp;
            const double smpso = g_par.pft.smpso[it], smpsc = g_par.pft.smpsc[it];
            if (io->h2osoi_liqvol[g] <= 0.0 || io->t_soisno[ss] <= TFRZ_ - 2.0) {
                io->rootr[pg] = 0.0;
            } else {
                const double s_node = std::max(io->h2osoi_liqvol[g] / io->eff_porosity[g], 0.01);
                double smp_node = -io->sucsat[g] * o_pow(s_node, -io->bsw[g]);
                smp_node = std::max(smpsc, smp_node);
                io->rresis[pg] = std::min((io->eff_porosity[g] / io->watsat[g]) * (smp_node - smpsc) / (smpso - smpsc), 1.0);
                io->rootr[pg] = io->rootfr[pg] * io->rresis[pg];
                io->btran[p] = io->btran[p] + std::max(io->rootr[pg], 0.0);
            }
        }
    for (int j = 1; j <= NLEVGRND_; ++j)
        for (int f = 0; f < nump; ++f) {
            const int p = filtp[f] - b->begp;
            const size_t pg = p + (size_t)(j - 1) * ldp;
            if (io->btran[p] > 0.0) io->rootr[pg] = io->rootr[pg] / io->btran[p];
            else io->rootr[pg] = 0.0;
        }
    return 0;
}

// BareGroundFluxes (src/biogeophys/BareGroundFluxesMod.F90:73-545) over
// filter_noexposedvegp, statement by statement; soil_resis_method 1 (sl_14,
// soilresis) or 0 (leepielke_1992, soilbeta).  The canopy parameters carry
// a_coef, a_exp, wind_min and zetamaxstable.
extern "C" int oracle_baregroundfluxes(const ctsmg_bounds* b, int nump, const int32_t* filtp,
                                       const ctsmg_baregrnd_io* io, int soil_resis_method) {
    const ctsmg_canopy_params& P = g_par.c;
    const double zii = 1000.0, beta = 1.0;
    const int ldp = io->ldp, ldc = io->ldc, LS_ = -CTSMG_NLEVSNO + 1;
    std::vector<double> zldis(nump), ur(nump), dth(nump), dqh(nump), obu(nump), um(nump), fm(nump);
    std::vector<FVOut> fvo(nump);
    auto PC = [&](int f) { return io->patch_column[filtp[f] - b->begp] - b->begc; };
    auto PG = [&](int f) { return io->patch_gridcell[filtp[f] - b->begp] - io->begg; };
    for (int f = 0; f < nump; ++f) {
        const int p = filtp[f] - b->begp, c = PC(f);
        io->btran[p] = 0.0;
        io->t_veg[p] = io->forc_t[c];
        const double cf_bare = io->forc_pbot[c] / (RGAS * 0.001 * io->thm[p]) * 1.e06;
        io->rssun[p] = 1.0 / 1.e15 * cf_bare;
        io->rssha[p] = 1.0 / 1.e15 * cf_bare;
        for (int j = 1; j <= CTSMG_NLEVGRND; ++j) {
            io->rootr[p + (size_t)(j - 1) * ldp] = 0.0;
            io->rresis[p + (size_t)(j - 1) * ldp] = 0.0;
        }
    }
    for (int f = 0; f < nump; ++f) {
        const int p = filtp[f] - b->begp, c = PC(f), g = PG(f);
        io->displa[p] = 0.0; io->z0mv[p] = 0.0; io->z0hv[p] = 0.0; io->z0qv[p] = 0.0;
        io->dlrad[p] = 0.0; io->ulrad[p] = 0.0; io->dhsdt_canopy[p] = 0.0; io->eflx_sh_stem[p] = 0.0;
        ur[f] = std::max(P.wind_min, std::sqrt(io->forc_u[g] * io->forc_u[g] + io->forc_v[g] * io->forc_v[g]));
        dth[f] = io->thm[p] - io->t_grnd[c];
        dqh[f] = io->forc_q[c] - io->qg[c];
        const double dthv = dth[f] * (1.0 + 0.61 * io->forc_q[c]) + 0.61 * io->forc_th[c] * dqh[f];
        zldis[f] = io->forc_hgt_u_patch[p];
        io->z0mg_patch[p] = io->z0mg[c];
        io->z0hg_patch[p] = io->z0hg[c];
        io->z0qg_patch[p] = io->z0qg[c];
        // MoninObukIni (FrictionVelocityMod.F90:1158-1209)
        const double wc = 0.5;
        if (dthv >= 0.0) um[f] = std::max(ur[f], 0.1);
        else um[f] = std::sqrt(ur[f] * ur[f] + wc * wc);
        const double rib = GRAV * zldis[f] * dthv / (io->thv[c] * um[f] * um[f]);
        double zeta;
        if (rib >= 0.0) {
            zeta = rib * o_log(zldis[f] / io->z0mg_patch[p]) / (1.0 - 5.0 * std::min(rib, 0.19));
            zeta = std::min(P.zetamaxstable, std::max(zeta, 0.01));
        } else {
            zeta = rib * o_log(zldis[f] / io->z0mg_patch[p]);
            zeta = std::max(-100.0, std::min(zeta, -0.01));
        }
        obu[f] = zldis[f] / zeta;
        io->num_iter[p] = 0;
    }
    for (int iter = 1; iter <= 3; ++iter) {
        for (int f = 0; f < nump; ++f) {
            const int p = filtp[f] - b->begp;
            friction_velocity(io->displa[p], io->z0mg_patch[p], io->z0hg_patch[p], io->z0qg_patch[p], obu[f], iter,
                              ur[f], um[f], io->forc_hgt_u_patch[p], io->forc_hgt_t_patch[p], io->forc_hgt_q_patch[p],
                              fm[f], fvo[f]);
        }
        for (int f = 0; f < nump; ++f) {
            const int p = filtp[f] - b->begp, c = PC(f), g = PG(f);
            const double ustar = fvo[f].ustar;
            const double tstar = fvo[f].temp1 * dth[f];
            const double qstar = fvo[f].temp2 * dqh[f];
            io->z0hg_patch[p] = io->z0mg_patch[p] / o_exp(P.a_coef * o_pow(ustar * io->z0mg_patch[p] / NU_PARAM, P.a_exp));
            io->z0qg_patch[p] = io->z0hg_patch[p];
            io->forc_hgt_u_patch[p] = io->forc_hgt_u[g] + io->z0mg_patch[p] + io->displa[p];
            io->forc_hgt_t_patch[p] = io->forc_hgt_t[g] + io->z0hg_patch[p] + io->displa[p];
            io->forc_hgt_q_patch[p] = io->forc_hgt_q[g] + io->z0qg_patch[p] + io->displa[p];
            const double thvstar = tstar * (1.0 + 0.61 * io->forc_q[c]) + 0.61 * io->forc_th[c] * qstar;
            double zeta = zldis[f] * VKC * GRAV * thvstar / (ustar * ustar * io->thv[c]);
            if (zeta >= 0.0) {
                zeta = std::min(P.zetamaxstable, std::max(zeta, 0.01));
                um[f] = std::max(ur[f], 0.1);
            } else {
                zeta = std::max(-100.0, std::min(zeta, -0.01));
                const double wc = beta * o_pow(-GRAV * ustar * thvstar * zii / io->thv[c], 0.333);
                um[f] = std::sqrt(ur[f] * ur[f] + wc * wc);
            }
            io->zeta[p] = zeta;
            obu[f] = zldis[f] / zeta;
            io->num_iter[p] = iter;
        }
    }
    for (int f = 0; f < nump; ++f) {
        const int p = filtp[f] - b->begp, c = PC(f), g = PG(f);
        const FVOut& o = fvo[f];
        io->obu[p] = obu[f]; io->fm[p] = fm[f];
        io->u10_clm[p] = o.u10_clm; io->u10[p] = o.u10; io->va[p] = o.va; io->vds[p] = o.vds; io->fv[p] = o.fv;
        const double ram = 1.0 / (o.ustar * o.ustar / um[f]);
        const double rah = 1.0 / (o.temp1 * o.ustar);
        const double raw = 1.0 / (o.temp2 * o.ustar);
        const double raih = io->forc_rho[c] * CPAIR / rah;
        double forc_qs, forc_esat;
        qsat(io->forc_t[c], io->forc_pbot[c], &forc_qs, &forc_esat, nullptr);
        const double forc_e = std::max((io->forc_q[c] * io->forc_pbot[c]) / (io->forc_q[c] + 0.622), 0.01 * forc_esat);
        const double t = io->t_grnd[c];
        double forc_dewpoint;            // dewpoint (:558-578)
        if (t < TFRZ) forc_dewpoint = 273.86 * o_log(forc_e / 611.21) / (22.587 - o_log(forc_e / 611.21));
        else forc_dewpoint = 243.04 * o_log(forc_e / 610.94) / (17.625 - o_log(forc_e / 610.94));
        forc_dewpoint = forc_dewpoint + TFRZ;
        double raiw = 0.0;
        if (dqh[f] > 0.0) {
            if (io->t_grnd[c] > forc_dewpoint) raiw = 0.0;
            else raiw = io->forc_rho[c] / raw;
        } else {
            if (soil_resis_method == 0) {
                if (io->t_grnd[c] > forc_dewpoint) raiw = 0.0;
                else raiw = io->soilbeta[c] * io->forc_rho[c] / raw;
            }
            if (soil_resis_method == 1) raiw = io->forc_rho[c] / (raw + io->soilresis[c]);
        }
        io->ram1[p] = ram;
        io->cgrnds[p] = raih;
        io->cgrndl[p] = raiw * io->dqgdT[c];
        io->cgrnd[p] = io->cgrnds[p] + io->htvp[c] * io->cgrndl[p];
        io->taux[p] = -io->forc_rho[c] * io->forc_u[g] / ram;
        io->tauy[p] = -io->forc_rho[c] * io->forc_v[g] / ram;
        io->eflx_sh_grnd[p] = -raih * dth[f];
        io->eflx_sh_tot[p] = io->eflx_sh_grnd[p];
        const int snl = io->snl[c];
        io->eflx_sh_snow[p] = -raih * (io->thm[p] - io->t_soisno[c + (size_t)(snl + 1 - LS_) * ldc]);
        io->eflx_sh_soil[p] = -raih * (io->thm[p] - io->t_soisno[c + (size_t)(1 - LS_) * ldc]);
        io->eflx_sh_h2osfc[p] = -raih * (io->thm[p] - io->t_h2osfc[c]);
        io->qflx_tran_veg[p] = 0.0;
        io->qflx_evap_veg[p] = 0.0;
        io->qflx_evap_soi[p] = -raiw * dqh[f];
        io->qflx_evap_tot[p] = io->qflx_evap_soi[p];
        io->qflx_ev_snow[p] = -raiw * (io->forc_q[c] - io->qg_snow[c]);
        io->qflx_ev_soil[p] = -raiw * (io->forc_q[c] - io->qg_soil[c]);
        io->qflx_ev_h2osfc[p] = -raiw * (io->forc_q[c] - io->qg_h2osfc[c]);
        io->t_ref2m[p] = io->thm[p] + o.temp1 * dth[f] * (1.0 / o.temp12m - 1.0 / o.temp1);
        io->q_ref2m[p] = io->forc_q[c] + o.temp2 * dqh[f] * (1.0 / o.temp22m - 1.0 / o.temp2);
        double qsat_ref2m, e_ref2m;
        qsat(io->t_ref2m[p], io->forc_pbot[c], &qsat_ref2m, &e_ref2m, nullptr);
        io->rh_ref2m[p] = std::min(100.0, io->q_ref2m[p] / qsat_ref2m * 100.0);
        io->kbm1[p] = o_log(io->z0mg_patch[p] / io->z0hg_patch[p]);
        io->z0hg[c] = io->z0hg_patch[p];
        io->z0qg[c] = io->z0qg_patch[p];
    }
    return 0;
}

