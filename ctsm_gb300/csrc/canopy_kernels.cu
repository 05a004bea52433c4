// canopy_kernels.cu -- sm_103a FP64 kernel for CanopyFluxes (leaf temperature
// / Monin-Obukhov stability iteration) with Photosynthesis sun + shade.
//
// Three kernels per call.  canopy_setup_kernel prepares every patch of the
// filter (CanopyFluxesMod.F90:700-1017) and writes its iteration state to a
// per-patch record in HBM.  canopy_iterate_kernel is persistent: one thread
// owns one patch at a time and runs its passes (:1028-1458); the reference
// removes converged patches from its filter after every pass (:1448-1456),
// and here a lane whose patch has converged (or reached itmax) stores the
// record and takes the next patch from a global work counter, then rejoins
// the warp for the next pass -- the GPU form of the reference's filter
// compaction.  canopy_finalize_kernel reads the records and computes the
// post-iteration fluxes (:1461-1655).  Keeping setup and finalize out of the
// iterating kernel keeps its code (one pass, one Ci root finder, one out-of-
// line copy of each libm function) small enough for the instruction cache,
// and its lanes never wait on another lane's setup or finalize.  Per-patch
// results do not depend on which lane or pass slot served them.
#include <cuda_runtime.h>
#include <cstdint>
#include "ctsm_device.cuh"
#include "fastmath.cuh"
#include "canopy_kernels.cuh"
#include "rootfind.cuh"
#include "qsat.cuh"
#include "fcmp.cuh"

namespace ctsmg {
namespace canopy {

constexpr double PI = 3.14159265358979323846;
constexpr double VKC = 0.4;
constexpr double CPAIR = 1.00464e3;
constexpr double HVAP = 2.501e6;
constexpr double RGAS = 6.02214e26 * 1.38065e-23;
constexpr double NU_PARAM = 1.5e-5;
constexpr double TLSAI_CRIT = 2.0;

__device__ __forceinline__ double ipow4(double x) { double x2 = x * x; return x2 * x2; }
__device__ __forceinline__ double ipow3(double x) { double x2 = x * x; return x2 * x; }

// Lane-occupancy probes for tuning builds (-DCTSMG_LANE_PROBE): per probe
// point, the number of warp-level executions and the sum of active lanes.
#ifdef CTSMG_LANE_PROBE
__device__ unsigned long long g_lane_probe[64];
#define LANE_PROBE(i)                                                                        \
    do {                                                                                     \
        const unsigned m_ = __activemask();                                                  \
        if ((int)(threadIdx.x & 31) == __ffs(m_) - 1) {                                      \
            atomicAdd(&g_lane_probe[2 * (i)], 1ull);                                         \
            atomicAdd(&g_lane_probe[2 * (i) + 1], (unsigned long long)__popc(m_));           \
        }                                                                                    \
    } while (0)
#else
#define LANE_PROBE(i) do {} while (0)
#endif

struct Err { int code, idx; };
__device__ __forceinline__ void flag(Err& e, int code, int idx) { if (!e.code) { e.code = code; e.idx = idx; } }

// quadraticMod.F90:17-74
__device__ __forceinline__ bool quadratic(double a, double b, double c, double& r1, double& r2) {
    if (!ic::ne0(a)) { r1 = r2 = 0.0; return false; }
    double root = b * b - 4.0 * a * c;
    if (ic::lt0(root)) {
        if (ic::gtn(root, -3.0 * 2.220446049250313e-16)) root = 0.0;
        else { r1 = r2 = 0.0; return false; }
    }
    const double q = ic::ge0(b) ? -0.5 * (b + sqrt(root)) : -0.5 * (b - sqrt(root));
    r1 = q / a;
    r2 = ic::ne0(q) ? c / q : 1.e36;
    return true;
}

// One out-of-line body of each libm function that the pass calls at several
// sites (FrictionVelocity, the stability functions, Photosynthesis): the
// iterating kernel holds one copy of each instead of an inline expansion per
// call site.  The functions are CUDA's own; only where their code sits changes.
__device__ __noinline__ double xlog(double x) { return fm::log(x); }
__device__ __noinline__ double xexp(double x) { return fm::exp(x); }
__device__ __noinline__ double xpow(double x, double y) { return fm::pow(x, y); }
__device__ __noinline__ double xatan(double x) { return atan(x); }

// FrictionVelocityMod.F90:1120-1155
__device__ __forceinline__ double stab1(double zeta) {
    const double chik2 = sqrt(1.0 - 16.0 * zeta);
    const double chik = sqrt(chik2);
    return 2.0 * xlog((1.0 + chik) * 0.5) + xlog((1.0 + chik2) * 0.5) - 2.0 * xatan(chik) + PI * 0.5;
}
__device__ __forceinline__ double stab2(double zeta) {
    return 2.0 * xlog((1.0 + sqrt(1.0 - 16.0 * zeta)) * 0.5);
}

struct PsnState { double ac, aj, ap, ag, an, gs_mol; };

// Inputs of ci_func for one patch and phase.  The ones that do not change
// while Ci is iterated are evaluated once, with the operations in the order
// ci_func writes them (kco = kc (1 + oair/ko), c14gb = 1.4/gb_mol, gbrh =
// gb_mol 1e-6 rh_can and the Medlyn constants).
struct PsnCtx {
    bool c3;
    int method;
    double vcmax_z, cp, kco, ap3, aj4, kp_z, theta_cj, theta_ip, forc_pbot;
    double m_slope, m_i6, m_i2_12, m_2i6, m_s;
    double bbb, mbb;
    double gb_mol, c14gb, gbrh, je, cair, lmr_z, rh_can;
};

// PhotosynthesisMod.F90:2564-2701
__device__ double ci_func(double ci, const PsnCtx& x, PsnState& s, Err& e, int pidx) {
    LANE_PROBE(4);
    double r1, r2;
    if (x.c3) {
        s.ac = x.vcmax_z * ic::max0(ci - x.cp) / (ci + x.kco);
        s.aj = x.je * ic::max0(ci - x.cp) / (4.0 * ci + 8.0 * x.cp);
        s.ap = x.ap3;
    } else {
        s.ac = x.vcmax_z;
        s.aj = x.aj4;
        s.ap = x.kp_z * ic::max0(ci) / x.forc_pbot;
    }
    if (!quadratic(x.theta_cj, -(s.ac + s.aj), s.ac * s.aj, r1, r2)) flag(e, CTSMG_E_DISCRIMINANT, pidx);
    const double ai = fmin(r1, r2);
    if (!quadratic(x.theta_ip, -(ai + s.ap), ai * s.ap, r1, r2)) flag(e, CTSMG_E_DISCRIMINANT, pidx);
    s.ag = ic::max0(fmin(r1, r2));
    s.an = s.ag - x.lmr_z;
    if (ic::lt0(s.an)) return 0.0;
    LANE_PROBE(5);
    double cs = x.cair - x.c14gb * s.an * x.forc_pbot;
    cs = ic::maxc(cs, 1.e-06);
    if (x.method == 1) {
        const double term = 1.6 * s.an / (cs / x.forc_pbot * 1.e06);
        const double st = x.m_slope * term;
        const double bquad = -(2.0 * (x.m_i6 + term) + st * st / x.gbrh);
        const double cquad = x.m_i2_12 + (x.m_2i6 + term * x.m_s) * term;
        if (!quadratic(1.0, bquad, cquad, r1, r2)) flag(e, CTSMG_E_DISCRIMINANT, pidx);
        s.gs_mol = fmax(r1, r2) * 1.e06;
    } else {
        const double bquad = cs * (x.gb_mol - x.bbb) - x.mbb * s.an * x.forc_pbot;
        const double cquad = -x.gb_mol * (cs * x.bbb + x.mbb * s.an * x.forc_pbot * x.rh_can);
        if (!quadratic(cs, bquad, cquad, r1, r2)) flag(e, CTSMG_E_DISCRIMINANT, pidx);
        s.gs_mol = fmax(r1, r2);
    }
    return ci - x.cair + s.an * x.forc_pbot * (1.4 * s.gs_mol + 1.6 * x.gb_mol) / (x.gb_mol * s.gs_mol);
}

__device__ __forceinline__ double ft(double tl, double ha) {
    return xexp(ha / (RGAS * 1.e-3 * (TFRZ + 25.0)) * (1.0 - (TFRZ + 25.0) / tl));
}
__device__ __forceinline__ double fth(double tl, double hd, double se, double sf) {
    return sf / (1.0 + xexp((-hd + se * tl) / (RGAS * 1.e-3 * tl)));
}
__device__ __forceinline__ double fth25(double hd, double se) {
    return 1.0 + xexp((-hd + se * (TFRZ + 25.0)) / (RGAS * 1.e-3 * (TFRZ + 25.0)));
}

struct PhaseOut { double rs, psn, lmr, ci, gs_mol_phase; };

// Photosynthesis quantities of a patch that stay fixed while CanopyFluxes
// iterates (PhotosynthesisMod.F90:1555-1830 with nlevcan = 1): canopy-top
// vcmax25 / jmax25, the acclimation entropies from the 10-day temperature,
// the high-temperature normalisers fth25, the conductance factor cf and the
// stomatal parameters.
struct PsnPatch {
    double vcmax25top, jmax25top, vcmaxse, jmaxse, tpuse, f25_lmr, f25_vc, f25_j, f25_tpu, cf, mslope, mint, mbb;
};

// Temperature factors of a pass: they depend on t_veg only, so the sunlit and
// shaded phases share them.  C3: ft and fth of lmr, vcmax, jmax, tpu; C4: the
// Q10 factor and the 1 + exp(...) divisors (PhotosynthesisMod.F90:1555-1562,
// 1722-1817).
struct PsnTemp { double kc, ko, cp, lmr1, lmr2, vc1, vc2, j1, j2, tpu1, tpu2, q10; };

// What a patch carries from setup to the passes and on to finalize, in two
// parts.  PatchK holds the quantities setup fixes for the whole iteration:
// the displaced heights and roughness, the wind, the longwave factors, the
// logarithms of the fixed heights over z0m in FrictionVelocity, (zetam)^0.333
// and (zetat)^-0.333, exp(-(elai+esai)), sqrt(dleaf), 1 - exp(-elai_dl), the
// ground's emitted longwave factor lw_grnd and the photosynthesis constants.
// The iterating kernel keeps it in shared memory, so that the registers hold
// only what the passes change.
struct PatchK {
    double displa, z0mv, hgt_u, hgt_t, hgt_q, zldis, ur, tl_ini, air, bir, cir, dayl_factor, liqcan, snocan;
    double lg_u, lg_u10, lg_t, lg_q, lg_2m, lg_u10m, pz_m, pz_t, s1_zetam, s2_zetat, w_sai, sqrt_dleaf, one_m_edl,
        lw_grnd;
    PsnPatch q;
};

// Patch holds what the passes change: the state carried from pass to pass and
// the last pass's values that finalize uses.
struct Patch {
    int p, c, g, ivt, itlef, nmozsgn, num_iter, c3, err_code, err_idx;
    double um, obu, obuold, fm;
    double t_veg, qsatl, el, qsatldT, taf, qaf, dth, dqh, delq;
    double del, efeb;
    // last-pass values used after the iteration
    double tlbef, dt_veg, err, eflx_sh_veg, qflx_evap_veg, qflx_tran_veg, lw_leaf, zeta;
    double ustar, temp1, temp2, temp12m, temp22m, ram1, rah_a, raw_a, rah_b, uaf, rb;
    double wtl0, wta0, wtg, wtal, wtgq, wtlq0, wtaq0, wtalq, efe;
    double u10_clm, u10, vds, vpd_can, rh_leaf, rhaf_last, vpd_last;
    PhaseOut sun, sha;
    PsnState st;
};

// The record of a patch in HBM: one plane per component, indexed by the
// patch's filter position (level-major like the model arrays).
#define PATCH_INTS(X) X(p) X(c) X(g) X(ivt) X(itlef) X(nmozsgn) X(num_iter) X(c3) X(err_code) X(err_idx)
#define PATCH_DOUBLES(X)                                                                                              \
    X(um) X(obu) X(obuold) X(fm)                                                                                      \
    X(t_veg) X(qsatl) X(el) X(qsatldT) X(taf) X(qaf) X(dth) X(dqh) X(delq)                                             \
    X(del) X(efeb)                                                                                                    \
    X(tlbef) X(dt_veg) X(err) X(eflx_sh_veg) X(qflx_evap_veg) X(qflx_tran_veg) X(lw_leaf) X(zeta)                     \
    X(ustar) X(temp1) X(temp2) X(temp12m) X(temp22m) X(ram1) X(rah_a) X(raw_a) X(rah_b) X(uaf) X(rb)                  \
    X(wtl0) X(wta0) X(wtg) X(wtal) X(wtgq) X(wtlq0) X(wtaq0) X(wtalq) X(efe)                                          \
    X(u10_clm) X(u10) X(vds) X(vpd_can) X(rh_leaf) X(rhaf_last) X(vpd_last)                                           \
    X(sun.rs) X(sun.psn) X(sun.lmr) X(sun.ci) X(sun.gs_mol_phase)                                                     \
    X(sha.rs) X(sha.psn) X(sha.lmr) X(sha.ci) X(sha.gs_mol_phase)                                                     \
    X(st.ac) X(st.aj) X(st.ap) X(st.ag) X(st.an) X(st.gs_mol)
#define PATCHK_DOUBLES(X)                                                                                             \
    X(displa) X(z0mv) X(hgt_u) X(hgt_t) X(hgt_q) X(zldis) X(ur) X(tl_ini) X(air) X(bir) X(cir) X(dayl_factor)          \
    X(liqcan) X(snocan)                                                                                               \
    X(lg_u) X(lg_u10) X(lg_t) X(lg_q) X(lg_2m) X(lg_u10m) X(pz_m) X(pz_t) X(s1_zetam) X(s2_zetat) X(w_sai)         \
    X(sqrt_dleaf) X(one_m_edl) X(lw_grnd)                                                                             \
    X(q.vcmax25top) X(q.jmax25top) X(q.vcmaxse) X(q.jmaxse) X(q.tpuse) X(q.f25_lmr) X(q.f25_vc) X(q.f25_j)            \
    X(q.f25_tpu) X(q.cf) X(q.mslope) X(q.mint) X(q.mbb)
#define PATCH_COUNT(m) +1
constexpr int NPI = 0 PATCH_INTS(PATCH_COUNT);
constexpr int NPV = 0 PATCH_DOUBLES(PATCH_COUNT);
constexpr int NPK = 0 PATCHK_DOUBLES(PATCH_COUNT);
constexpr int NPD = NPV + NPK;                // double planes of the record: Patch's, then PatchK's
static_assert(sizeof(Patch) == NPI * 4 + NPV * 8, "every Patch component must be listed in PATCH_INTS / PATCH_DOUBLES");
static_assert(sizeof(PatchK) == NPK * 8, "every PatchK component must be listed in PATCHK_DOUBLES");

__device__ __forceinline__ void store_patch(double* ws, int ld, int f, const Patch& s) {
    int* wi = reinterpret_cast<int*>(ws + (size_t)NPD * ld);
    int k = 0;
#define ST_D(m) ws[(size_t)(k++) * ld + f] = s.m;
    PATCH_DOUBLES(ST_D)
#undef ST_D
    k = 0;
#define ST_I(m) wi[(size_t)(k++) * ld + f] = s.m;
    PATCH_INTS(ST_I)
#undef ST_I
}

__device__ __forceinline__ void store_patchk(double* ws, int ld, int f, const PatchK& s) {
    int k = NPV;
#define ST_K(m) ws[(size_t)(k++) * ld + f] = s.m;
    PATCHK_DOUBLES(ST_K)
#undef ST_K
}

__device__ __forceinline__ void load_patchk(const double* __restrict__ ws, int ld, int f, PatchK& s) {
    int k = NPV;
#define LD_K(m) s.m = ws[(size_t)(k++) * ld + f];
    PATCHK_DOUBLES(LD_K)
#undef LD_K
}

__device__ __forceinline__ void load_patch(const double* __restrict__ ws, int ld, int f, Patch& s) {
    const int* wi = reinterpret_cast<const int*>(ws + (size_t)NPD * ld);
    int k = 0;
#define LD_D(m) s.m = ws[(size_t)(k++) * ld + f];
    PATCH_DOUBLES(LD_D)
#undef LD_D
    k = 0;
#define LD_I(m) s.m = wi[(size_t)(k++) * ld + f];
    PATCH_INTS(LD_I)
#undef LD_I
}

// PhotosynthesisMod.F90:1555-1830: the factors of the pass's t_veg.  The
// day-time ones (kc, ko, cp, vcmax, jmax, tpu) only when a phase has light.
__device__ void psn_temp(const CanopyArgs& A, const Patch& s, const PatchK& K, double forc_pbot, double oair, bool day, PsnTemp& T) {
    const ctsmg_canopy_params& P = A.par;
    const double t_veg = s.t_veg;
    if (s.c3) {
        T.lmr1 = ft(t_veg, P.lmrha);
        T.lmr2 = fth(t_veg, P.lmrhd, P.lmrse, K.q.f25_lmr);
    } else {
        T.q10 = xpow(2.0, (t_veg - (TFRZ + 25.0)) / 10.0);
        T.lmr2 = 1.0 + xexp(1.3 * (t_veg - (TFRZ + 55.0)));
    }
    if (!day) return;
    LANE_PROBE(6);
    T.kc = P.kc25_coef * forc_pbot * ft(t_veg, P.kcha);
    T.ko = P.ko25_coef * forc_pbot * ft(t_veg, P.koha);
    const double sco = 0.5 * 0.209 / P.cp25_yr2000;
    T.cp = 0.5 * oair / sco * ft(t_veg, P.cpha);
    if (s.c3) {
        T.vc1 = ft(t_veg, P.vcmaxha);
        T.vc2 = fth(t_veg, P.vcmaxhd, K.q.vcmaxse, K.q.f25_vc);
    } else {
        T.vc1 = 1.0 + xexp(0.2 * ((TFRZ + 15.0) - t_veg));
        T.vc2 = 1.0 + xexp(0.3 * (t_veg - (TFRZ + 40.0)));
    }
    T.j1 = ft(t_veg, P.jmaxha);
    T.j2 = fth(t_veg, P.jmaxhd, K.q.jmaxse, K.q.f25_j);
    T.tpu1 = ft(t_veg, P.tpuha);
    T.tpu2 = fth(t_veg, P.tpuhd, K.q.tpuse, K.q.f25_tpu);
}

// PhotosynthesisMod.F90:1243-2062, one phase, nlevcan = nrad = 1
__device__ PhaseOut photosynthesis(const CanopyArgs& A, const Patch& s, const PatchK& K, const PsnTemp& T, int pidx, double forc_pbot,
                                   double esat_tv, double eair, double oair, double cair, double rb, double btran,
                                   double par_z, double lai_z, double vcmaxcint, PsnState& st, double& vpd_can,
                                   double& rh_leaf, Err& err) {
    const ctsmg_canopy_params& P = A.par;
    const int method = A.method;
    LANE_PROBE(3);
    const PsnPatch& q = K.q;
    const double medlyn_int = q.mint;
    const bool c3 = s.c3 != 0;
    const double qe = c3 ? 0.0 : 0.05;
    double bbb = 0.0, mbb = 0.0;
    if (method == 0) { bbb = ic::maxc((c3 ? 10000.0 : 40000.0) * btran, 1.0); mbb = q.mbb; }
    const double nscaler = vcmaxcint;
    const double lmr25 = (c3 ? q.vcmax25top * P.leaf_mr_vcm : q.vcmax25top * 0.025) * nscaler;
    double lmr_z;
    if (c3) {
        lmr_z = lmr25 * T.lmr1 * T.lmr2;
    } else {
        lmr_z = lmr25 * T.q10;
        lmr_z = lmr_z / T.lmr2;
    }
    double vcmax_z = 0.0, jmax_z = 0.0, tpu_z = 0.0, kp_z = 0.0;
    if (ic::gt0(par_z)) {
        const double vcmax25 = q.vcmax25top * nscaler, jmax25 = q.jmax25top * nscaler;
        const double tpu25 = P.tpu25ratio * q.vcmax25top * nscaler, kp25 = P.kp25ratio * q.vcmax25top * nscaler;
        if (c3) {
            vcmax_z = vcmax25 * T.vc1 * T.vc2;
        } else {
            vcmax_z = vcmax25 * T.q10;
            vcmax_z = vcmax_z / T.vc1;
            vcmax_z = vcmax_z / T.vc2;
            kp_z = kp25 * T.q10;
        }
        jmax_z = jmax25 * T.j1 * T.j2;
        tpu_z = tpu25 * T.tpu1 * T.tpu2;
    }
    vcmax_z = vcmax_z * btran;
    lmr_z = lmr_z * btran;
    if (P.light_inhibit && ic::gt0(par_z)) lmr_z = lmr_z * 0.67;

    const double rsmax0 = 2.e4;
    const double cf = q.cf;
    const double gb_mol = 1.0 / rb * cf;
    PhaseOut out;
    double rs_z, psn_z, ci_z;
    if (ic::le0(par_z)) {
        st.ac = st.aj = st.ap = st.ag = 0.0;
        st.an = 0.0 - lmr_z;
        psn_z = 0.0;
        rs_z = (method == 0) ? ic::minc(1.0 / bbb * cf, rsmax0) : ic::minc(1.0 / medlyn_int * cf, rsmax0);
        ci_z = 0.0;
        rh_leaf = 0.0;
        out.gs_mol_phase = cf / rs_z;
    } else {
        const double ceair = fmin(eair, esat_tv);
        double rh_can;
        if (method == 0) {
            rh_can = ceair / esat_tv;
        } else {
            rh_can = ic::maxc((esat_tv - ceair), 50.0) * 0.001;
            vpd_can = rh_can;
        }
        const double qabs = 0.5 * (1.0 - P.fnps) * par_z * 4.6;
        double r1, r2;
        if (!quadratic(P.theta_psii, -(qabs + jmax_z), qabs * jmax_z, r1, r2)) flag(err, CTSMG_E_DISCRIMINANT, pidx);
        const double ms = q.mslope, mi = medlyn_int;
        const PsnCtx ctx{c3, method, vcmax_z, T.cp, T.kc * (1.0 + oair / T.ko), 3.0 * tpu_z, qe * par_z * 4.6, kp_z,
                         A.pft.theta_cj[s.ivt], P.theta_ip, forc_pbot,
                         ms, mi * 1.e-06, mi * mi * 1.e-12, 2.0 * mi * 1.e-06, 1.0 - ms * ms / rh_can,
                         bbb, mbb, gb_mol, 1.4 / gb_mol, gb_mol * 1.e-06 * rh_can, fmin(r1, r2), cair, lmr_z, rh_can};
        RootFind rf;                                   // hybrid + brent, one evaluation site
        rf.start(c3 ? 0.7 * cair : 0.4 * cair);
#pragma unroll 1
        while (rf.next(ci_func(rf.x, ctx, st, err, pidx))) {}
        if (rf.not_bracketed) flag(err, CTSMG_E_NOT_BRACKETED, pidx);
        if (ic::lt0(st.an)) st.gs_mol = (method == 0) ? bbb : medlyn_int;
        out.gs_mol_phase = st.gs_mol;
        ci_z = cair - st.an * forc_pbot * (1.4 * st.gs_mol + 1.6 * gb_mol) / (gb_mol * st.gs_mol);
        ci_z = ic::maxc(ci_z, 1.e-06);
        rs_z = ic::minc(1.0 / (st.gs_mol / cf), rsmax0);
        psn_z = st.ag;
        if (ic::lt0(st.gs_mol)) flag(err, CTSMG_E_ARG, pidx);
        if (method == 0) rh_leaf = (gb_mol * ceair + st.gs_mol * esat_tv) / ((gb_mol + st.gs_mol) * esat_tv);
    }
    if (ic::gt0(lai_z)) {
        out.psn = psn_z * lai_z / lai_z;
        out.lmr = lmr_z * lai_z / lai_z;
        out.rs = lai_z / (lai_z / (rb + rs_z)) - rb;
    } else {
        out.psn = 0.0; out.lmr = 0.0; out.rs = 0.0;
    }
    out.ci = ci_z;
    return out;
}

// FrictionVelocityMod.F90:754-1117 for one patch (z0h = z0q = z0m), with the
// logarithms of the fixed heights taken from the patch record.
__device__ void friction_velocity(const Patch& s, const PatchK& K, int iter, double& fm, double& ustar, double& temp1, double& temp2,
                                  double& temp12m, double& temp22m, double& u10_clm, double& u10, double& vds) {
    const double zetam = 1.574, zetat = 0.465;
    const double obu = s.obu, z0m = K.z0mv, um = s.um;
    double zldis = K.hgt_u - K.displa;
    double zeta = zldis / obu;
    LANE_PROBE(1);
    // The momentum and scalar profiles each take one of four stability
    // branches, and a warp's lanes are often in different ones.  Every
    // logarithm, power and stability function the branches need is formed
    // once per warp in a "slot" whose argument each lane selects for its own
    // branch, then the branches combine the slots' values: the arguments and
    // the arithmetic are the reference's, only the control flow differs.
    const bool b1 = ic::ltn(zeta, -zetam), b2 = !b1 && ic::lt0(zeta), b3 = !b1 && !b2 && ic::lec(zeta, 1.0);
    const bool b4 = !b1 && !b2 && !b3;
    const bool tall = !ic::lec(zldis - z0m, 10.0);
    const double z10 = 10.0 + z0m;
    // the scalar profiles' heights and their branches (z0 = z0m in every call)
    const bool two = !(K.hgt_q == K.hgt_t);
    const double zl[3] = {K.hgt_t - K.displa, two ? K.hgt_q - K.displa : 0.0, 2.0 + K.z0mv};
    double zt[3];
    int tb[3];                      // 1..4: zt < -zetat, zt < 0, zt <= 1, else
    bool any_t1 = false, any_t4 = false;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        zt[i] = zl[i] / obu;
        tb[i] = ic::ltn(zt[i], -zetat) ? 1 : ic::lt0(zt[i]) ? 2 : ic::lec(zt[i], 1.0) ? 3 : 4;
        if (i == 1 && !two) tb[i] = 0;
        any_t1 |= tb[i] == 1;
        any_t4 |= tb[i] == 4;
    }
    // slots shared by the branches
    double pz = 0.0, s2z0 = 0.0, st_z0 = 0.0, st_zeta = 0.0, st_z10 = 0.0, l_a = 0.0, l_b = 0.0, l_zeta = 0.0;
    double l_t1 = 0.0, p_vds = 0.0;
    if (b1) pz = xpow(-zeta, 0.333);
    if (ic::lt0(obu)) s2z0 = stab2(z0m / obu);
    if (b1 || b2) st_z0 = stab1(z0m / obu);
    if (b2) st_zeta = stab1(zeta);
    if ((b1 || b2) && tall) st_z10 = stab1(z10 / obu);
    if (b1 || b4 || any_t4) l_a = xlog(b1 ? -zetam * obu / z0m : obu / z0m);     // b1: ustar; else log(obu / z0m)
    if ((b1 || b4) && tall) l_b = xlog(b1 ? -zetam * obu / z10 : obu / z10);
    if (b4) l_zeta = xlog(zeta);
    if (any_t1) l_t1 = xlog(-zetat * obu / z0m);
    // log(obu / z0m) for a scalar branch 4 of a lane whose momentum branch
    // took slot l_a for branch 1 (zl and zldis of opposite signs)
    double l_obu = l_a;
    if (b1 && any_t4) l_obu = xlog(obu / z0m);
    if (ic::lt0(zeta)) p_vds = xpow(300.0 / (-obu), 0.666);
    LANE_PROBE(8);
    if (b1) ustar = VKC * um / (l_a - K.s1_zetam + st_z0 + 1.14 * (pz - K.pz_m));
    else if (b2) ustar = VKC * um / (K.lg_u - st_zeta + st_z0);
    else if (b3) ustar = VKC * um / (K.lg_u + 5.0 * zeta - 5.0 * z0m / obu);
    else ustar = VKC * um / (l_a + 5.0 - 5.0 * z0m / obu + (5.0 * l_zeta + zeta - 1.0));
    vds = ic::lt0(zeta) ? 2.e-3 * ustar * (1.0 + p_vds) : 2.e-3 * ustar;
    if (!tall) {
        u10_clm = um;
    } else if (b1) {
        u10_clm = um - (ustar / VKC * (l_b - K.s1_zetam + st_z10 + 1.14 * (pz - K.pz_m)));
    } else if (b2) {
        u10_clm = um - (ustar / VKC * (K.lg_u10 - st_zeta + st_z10));
    } else if (b3) {
        u10_clm = um - (ustar / VKC * (K.lg_u10 + 5.0 * zeta - 5.0 * z10 / obu));
    } else {
        u10_clm = um - (ustar / VKC * (l_b + 5.0 - 5.0 * z10 / obu + (5.0 * l_zeta + zeta - 1.0)));
    }
    // scalar profiles: per call one power slot (branch 1) and one logarithm
    // slot (branch 2: stab2's logarithm; branch 4: log(zt))
    const double lgz[3] = {K.lg_t, K.lg_q, K.lg_2m};
    double tp[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int b = tb[i];
        const double z = zt[i];
        double pw = 0.0, lg = 0.0;
        if (b == 1) pw = xpow(-z, -0.333);
        if (b == 2 || b == 4) lg = xlog(b == 2 ? (1.0 + sqrt(1.0 - 16.0 * z)) * 0.5 : z);
        if (b == 1) tp[i] = VKC / (l_t1 - K.s2_zetat + s2z0 + 0.8 * (K.pz_t - pw));
        else if (b == 2) tp[i] = VKC / (lgz[i] - 2.0 * lg + s2z0);
        else if (b == 3) tp[i] = VKC / (lgz[i] + 5.0 * z - 5.0 * z0m / obu);
        else tp[i] = VKC / (l_obu + 5.0 - 5.0 * z0m / obu + (5.0 * lg + z - 1.0));
    }
    temp1 = tp[0];
    temp2 = two ? tp[1] : temp1;                  // z0qv == z0hv here
    temp12m = tp[2];
    temp22m = temp12m;
    double fmnew;
    LANE_PROBE(2);
    const double zeta1 = ic::minc(zeta, 1.0);
    if (ic::lt0(zeta1)) {
        LANE_PROBE(11);
        const double tmp1 = xpow(1.0 - 16.0 * zeta1, 0.25);
        fmnew = 2.0 * xlog((1.0 + tmp1) / 2.0) + xlog((1.0 + tmp1 * tmp1) / 2.0) - 2.0 * xatan(tmp1) + 1.5707963;
    } else {
        fmnew = -5.0 * zeta1;
    }
    fm = (iter == 1) ? fmnew : 0.5 * (fm + fmnew);
    double zeta10 = ic::minc(10.0 / obu, 1.0);
    if (!ic::ne0(zeta)) zeta10 = 0.0;
    double fm10;
    if (ic::lt0(zeta10)) {
        const double tmp1 = xpow(1.0 - 16.0 * zeta10, 0.25);
        fm10 = 2.0 * xlog((1.0 + tmp1) / 2.0) + xlog((1.0 + tmp1 * tmp1) / 2.0) - 2.0 * xatan(tmp1) + 1.5707963;
    } else {
        fm10 = -5.0 * zeta10;
    }
    u10 = K.ur - ustar / VKC * (K.lg_u10m - fm + fm10);
}

__device__ void setup(const CanopyArgs& A, Patch& s, PatchK& K, int p, Err& err) {
    const ctsmg_canopy_io& io = A.io;
    s.p = p;
    s.c = io.patch_column[p] - A.begc;
    s.g = io.patch_gridcell[p] - io.begg;
    s.ivt = io.itype[p];
    const int c = s.c, g = s.g;
    const double elai = io.elai[p], esai = io.esai[p], emv = io.emv[p], emg = io.emg[c];
    s.del = 0.0; s.efeb = 0.0; s.obuold = 0.0;
    s.wtgq = 0.0; s.wtlq0 = 0.0; s.wtaq0 = 0.0; s.wtalq = 0.0;
    K.dayl_factor = fmin(1.0, fmax(0.01, (io.dayl[g] * io.dayl[g]) / (io.max_dayl[g] * io.max_dayl[g])));
    io.rb1[p] = 0.0;
    const double lt = fmin(elai + esai, TLSAI_CRIT);
    const double egvf = (1.0 - xexp(-lt)) / (1.0 - xexp(-TLSAI_CRIT));
    K.displa = egvf * io.displa[p];
    K.z0mv = xexp(egvf * xlog(io.z0mv[p]) + (1.0 - egvf) * xlog(io.z0mg[c]));
    K.hgt_u = io.forc_hgt_u[g] + K.z0mv + K.displa;
    K.hgt_t = io.forc_hgt_t[g] + K.z0mv + K.displa;
    K.hgt_q = io.forc_hgt_q[g] + K.z0mv + K.displa;
    K.air = emv * (1.0 + (1.0 - emv) * (1.0 - emg)) * io.forc_lwrad[c];
    K.bir = -(2.0 - emv * (1.0 - emg)) * emv * SB;
    K.cir = emv * emg * SB;
    s.t_veg = io.t_veg[p];
    qsat(s.t_veg, io.forc_pbot[c], s.qsatl, s.el, &s.qsatldT);
    s.nmozsgn = 0;
    const double thm = io.thm[p], forc_q = io.forc_q[c], qg = io.qg[c];
    s.taf = (io.t_grnd[c] + thm) / 2.0;
    s.qaf = (forc_q + qg) / 2.0;
    K.ur = fmax(A.par.wind_min, sqrt(io.forc_u[g] * io.forc_u[g] + io.forc_v[g] * io.forc_v[g]));
    s.dth = thm - s.taf;
    s.dqh = forc_q - s.qaf;
    s.delq = qg - s.qaf;
    const double dthv = s.dth * (1.0 + 0.61 * forc_q) + 0.61 * io.forc_th[c] * s.dqh;
    K.zldis = K.hgt_u - K.displa;
    if (K.zldis < 0.0) flag(err, CTSMG_E_FORCING_HEIGHT, p + A.begp);
    const double thv = io.thv[c];
    s.um = (dthv >= 0.0) ? fmax(K.ur, 0.1) : sqrt(K.ur * K.ur + 0.5 * 0.5);
    const double rib = GRAV * K.zldis * dthv / (thv * s.um * s.um);
    double zeta;
    if (rib >= 0.0) {
        zeta = rib * xlog(K.zldis / K.z0mv) / (1.0 - 5.0 * fmin(rib, 0.19));
        zeta = fmin(A.par.zetamaxstable, fmax(zeta, 0.01));
    } else {
        zeta = rib * xlog(K.zldis / K.z0mv);
        zeta = fmax(-100.0, fmin(zeta, -0.01));
    }
    s.obu = K.zldis / zeta;
    // fixed during the iteration: FrictionVelocity's logarithms of the
    // heights over z0m, the pass's vegetation / snow factors, lw_grnd
    K.lg_u = xlog(K.zldis / K.z0mv);
    K.lg_u10 = xlog(K.zldis / (10.0 + K.z0mv));
    K.lg_t = xlog((K.hgt_t - K.displa) / K.z0mv);
    K.lg_q = xlog((K.hgt_q - K.displa) / K.z0mv);
    K.lg_2m = xlog((2.0 + K.z0mv) / K.z0mv);
    K.lg_u10m = xlog(fmax(1.0, K.hgt_u / 10.0));
    K.pz_m = xpow(1.574, 0.333);
    K.pz_t = xpow(0.465, -0.333);
    K.s1_zetam = stab1(-1.574);
    K.s2_zetat = stab2(-0.465);
    K.w_sai = xexp(-(elai + esai));
    K.sqrt_dleaf = sqrt(A.pft.dleaf[s.ivt]);
    {
        const double fsno_dl = io.snow_depth[c] / A.par.z_dl;
        const double elai_dl = A.par.lai_dl * (1.0 - fmin(fsno_dl, 1.0));
        K.one_m_edl = 1.0 - xexp(-elai_dl);
        const int ldc = io.ldc, snl = io.snl[c];
        const double frac_sno = io.frac_sno_eff[c], frac_h2osfc = io.frac_h2osfc[c];
        K.lw_grnd = (frac_sno * ipow4(io.t_soisno[c + (size_t)(snl + NLEVSNO) * ldc]) +
                     (1.0 - frac_sno - frac_h2osfc) * ipow4(io.t_soisno[c + (size_t)NLEVSNO * ldc]) +
                     frac_h2osfc * ipow4(io.t_h2osfc[c]));
    }
    // Photosynthesis constants of the patch (PhotosynthesisMod.F90:1555-1830)
    {
        const ctsmg_canopy_params& P = A.par;
        const ctsmg_pftcon& F = A.pft;
        const int ivt = s.ivt;
        s.c3 = (llround(F.c3psn[ivt]) == 1) ? 1 : 0;
        const double lnc = 1.0 / (F.slatop[ivt] * F.leafcn[ivt]);
        double vcmax25top = lnc * F.flnr[ivt] * P.fnr * P.act25 * K.dayl_factor;
        vcmax25top = vcmax25top * F.fnitr[ivt];
        const double t10c = fmin(fmax((io.t_a10[p] - TFRZ), 11.0), 35.0);
        K.q.vcmax25top = vcmax25top;
        K.q.jmax25top = ((2.59 - 0.035 * t10c) * vcmax25top) * P.jmax25top_sf;
        K.q.vcmaxse = (668.39 - 1.07 * t10c) * P.vcmaxse_sf;
        K.q.jmaxse = (659.70 - 0.75 * t10c) * P.jmaxse_sf;
        K.q.tpuse = (668.39 - 1.07 * t10c) * P.tpuse_sf;
        K.q.f25_lmr = fth25(P.lmrhd, P.lmrse);
        K.q.f25_vc = fth25(P.vcmaxhd, K.q.vcmaxse);
        K.q.f25_j = fth25(P.jmaxhd, K.q.jmaxse);
        K.q.f25_tpu = fth25(P.tpuhd, K.q.tpuse);
        K.q.cf = io.forc_pbot[c] / (RGAS * 1.e-3 * thm) * 1.e06;
        K.q.mslope = A.medlynslope_p ? A.medlynslope_p[p] : F.medlynslope[ivt];
        K.q.mint = A.medlynintercept_p ? A.medlynintercept_p[p] : F.medlynintercept[ivt];
        K.q.mbb = F.mbbopt[ivt];
    }
    s.num_iter = 0;
    K.tl_ini = s.t_veg;
    K.liqcan = io.liqcan[p];
    K.snocan = io.snocan[p];
    s.fm = 0.0;
    s.itlef = 0;
    s.st = PsnState{0, 0, 0, 0, 0, 0};
    s.vpd_can = 0.0;
    s.rh_leaf = 0.0;
}

// one pass of the stability iteration (CanopyFluxesMod.F90:1028-1456);
// returns true when the patch leaves the iteration
__device__ bool pass(const CanopyArgs& A, Patch& s, const PatchK& K, Err& err, double dtime) {
    const ctsmg_canopy_io& io = A.io;
    const ctsmg_canopy_params& P = A.par;
    const int p = s.p, c = s.c, g = s.g;
    const int pg = p + A.begp;
    LANE_PROBE(0);
    friction_velocity(s, K, s.itlef + 1, s.fm, s.ustar, s.temp1, s.temp2, s.temp12m, s.temp22m, s.u10_clm, s.u10, s.vds);
    const double ustar = s.ustar;
    s.tlbef = s.t_veg;
    const double del2 = s.del;
    s.ram1 = 1.0 / (ustar * ustar / s.um);
    s.rah_a = 1.0 / (s.temp1 * ustar);
    s.raw_a = 1.0 / (s.temp2 * ustar);
    s.uaf = s.um * sqrt(1.0 / (s.ram1 * s.um));
    const double elai = io.elai[p], esai = io.esai[p];
    const double cfl = P.cv / (sqrt(s.uaf) * K.sqrt_dleaf);
    s.rb = 1.0 / (cfl * s.uaf);
    const double rb = s.rb;
    const double w = K.w_sai;
    const double csoilb = VKC / (P.a_coef * xpow(io.z0mg[c] * s.uaf / NU_PARAM, P.a_exp));
    const double csoilcn = csoilb * w + P.csoilc * (1.0 - w);
    s.rah_b = 1.0 / (csoilcn * s.uaf);
    const double raw_b = s.rah_b;
    const double forc_pbot = io.forc_pbot[c];
    const double svpts = s.el;
    const double eah = forc_pbot * s.qaf / 0.622;
    s.rhaf_last = eah / svpts;
    s.vpd_last = ic::maxc((svpts - eah), 50.0) * 0.001;
    const double thm = io.thm[p], btran = io.btran[p];
    const double laisun = io.laisun[p], laisha = io.laisha[p];
    const double oair = io.forc_po2[g], cair = io.forc_pco2[g];
    const double parsun = io.parsun_z[p], parsha = io.parsha_z[p];
    PsnTemp T;
    psn_temp(A, s, K, forc_pbot, oair, ic::gt0(parsun) || ic::gt0(parsha), T);
    // sunlit then shaded phase (PhotosynthesisMod called with phase='sun' and
    // 'sha', CanopyFluxesMod.F90:1143-1169); a loop, so the phase body and
    // its root finder are compiled once
#pragma unroll 1
    for (int ph = 0; ph < 2; ++ph) {
        const PhaseOut o = photosynthesis(A, s, K, T, pg, forc_pbot, svpts, eah, oair, cair, rb, btran,
                                          ph ? parsha : parsun, ph ? laisha : laisun,
                                          ph ? io.vcmaxcintsha[p] : io.vcmaxcintsun[p], s.st, s.vpd_can, s.rh_leaf,
                                          err);
        if (ph) s.sha = o;
        else s.sun = o;
    }
    LANE_PROBE(7);
    const double sa_leaf = elai + esai;
    const double wta = 1.0 / s.rah_a;
    const double wtl = sa_leaf / rb;
    s.wtg = 1.0 / s.rah_b;
    const double wtshi = 1.0 / (wta + wtl + 0.0 + s.wtg);
    s.wtl0 = wtl * wtshi;
    const double wtg0 = s.wtg * wtshi;
    s.wta0 = wta * wtshi;
    const double wtga = s.wta0 + wtg0 + 0.0;
    s.wtal = s.wta0 + s.wtl0 + 0.0;
    const double fdry = io.fdry[p], fwet = io.fwet[p];
    const double rppdry = ic::gt0(fdry) ? fdry * rb * (laisun / (rb + s.sun.rs) + laisha / (rb + s.sha.rs)) / elai : 0.0;
    const double forc_rho = io.forc_rho[c], forc_q = io.forc_q[c], qg = io.qg[c], t_grnd = io.t_grnd[c];
    double efpot = forc_rho * ((elai + esai) / rb) * (s.qsatl - s.qaf);
    const double h2ocan = K.liqcan + K.snocan;
    double rpp;
    if (ic::gt0(efpot)) {
        if (ic::gt0(btran)) { s.qflx_tran_veg = efpot * rppdry; rpp = rppdry + fwet; }
        else { rpp = fwet; s.qflx_tran_veg = 0.0; }
        rpp = fmin(rpp, (s.qflx_tran_veg + h2ocan / dtime) / efpot);
    } else {
        rpp = 1.0;
        s.qflx_tran_veg = 0.0;
    }
    const double fv = fm::i2d(io.frac_veg_nosno[p]);
    const double wtaq = fv / s.raw_a;
    const double wtlq = fv * (elai + esai) / rb * rpp;
    const double rdl = K.one_m_edl / (0.004 * s.uaf);
    s.wtgq = ic::lt0(s.delq) ? fv / (raw_b + rdl) : fv / (raw_b + io.soilresis[c]);
    const double wtsqi = 1.0 / (wtaq + wtlq + s.wtgq);
    const double wtgq0 = s.wtgq * wtsqi;
    s.wtlq0 = wtlq * wtsqi;
    s.wtaq0 = wtaq * wtsqi;
    const double wtgaq = s.wtaq0 + wtgq0;
    s.wtalq = s.wtaq0 + s.wtlq0;
    const double dc1 = forc_rho * CPAIR * wtl;
    const double dc2 = HVAP * forc_rho * wtlq;
    const double efsh = dc1 * (wtga * s.t_veg - wtg0 * t_grnd - s.wta0 * thm - 0.0);
    s.efe = dc2 * (wtgaq * s.qsatl - wtgq0 * qg - s.wtaq0 * forc_q);
    double erre = 0.0;
    if (ic::lt0(s.efe * s.efeb)) {
        const double efeold = s.efe;
        s.efe = 0.1 * efeold;
        erre = s.efe - efeold;
    }
    const double lw_grnd = K.lw_grnd;
    const double sabv = io.sabv[p];
    const double t_veg = s.t_veg;
    double dt_veg = ((1.0 - 0.0) * (sabv + K.air + K.bir * ipow4(t_veg) + K.cir * lw_grnd) - efsh - s.efe - 0.0 + 0.0 -
                     (0.0 / dtime) * (t_veg - K.tl_ini)) /
                    ((1.0 - 0.0) * (-4.0 * K.bir * ipow3(t_veg)) + 4.0 * 0.0 * io.emv[p] * SB * ipow3(t_veg) + dc1 * wtga +
                     dc2 * wtgaq * s.qsatldT + 0.0 / dtime);
    s.t_veg = s.tlbef + dt_veg;
    const double dels = dt_veg;
    s.del = fabs(dels);
    s.err = 0.0;
    if (ic::gtc(s.del, 1.0)) {
        dt_veg = 1.0 * dels / s.del;
        s.t_veg = s.tlbef + dt_veg;
        const double tb3 = ipow3(s.tlbef);
        s.err = (1.0 - 0.0) * (sabv + K.air + K.bir * tb3 * (s.tlbef + 4.0 * dt_veg) + K.cir * lw_grnd) -
                0.0 * io.emv[p] * SB * tb3 * (s.tlbef + 4.0 * dt_veg) + 0.0 - (efsh + dc1 * wtga * dt_veg) -
                (s.efe + dc2 * wtgaq * s.qsatldT * dt_veg) - (0.0 / dtime) * (s.t_veg - K.tl_ini);
    }
    s.dt_veg = dt_veg;
    efpot = forc_rho * ((elai + esai) / rb) * (wtgaq * (s.qsatl + s.qsatldT * dt_veg) - wtgq0 * qg - s.wtaq0 * forc_q);
    s.qflx_evap_veg = rpp * efpot;
    s.qflx_tran_veg = (ic::gt0(efpot) && ic::gt0(btran)) ? efpot * rppdry : 0.0;
    const double ecidif = ic::max0(s.qflx_evap_veg - s.qflx_tran_veg - h2ocan / dtime);
    s.qflx_evap_veg = fmin(s.qflx_evap_veg, s.qflx_tran_veg + h2ocan / dtime);
    s.eflx_sh_veg = efsh + dc1 * wtga * dt_veg + s.err + erre + HVAP * ecidif;
    s.lw_leaf = 0.0 * io.emv[p] * SB * ipow3(s.tlbef) * (s.tlbef + 4.0 * dt_veg);
    qsat(s.t_veg, forc_pbot, s.qsatl, s.el, &s.qsatldT);
    s.taf = wtg0 * t_grnd + s.wta0 * thm + s.wtl0 * s.t_veg + 0.0;
    s.qaf = s.wtlq0 * s.qsatl + wtgq0 * qg + forc_q * s.wtaq0;
    s.dth = thm - s.taf;
    s.dqh = forc_q - s.qaf;
    s.delq = s.wtalq * qg - s.wtlq0 * s.qsatl - s.wtaq0 * forc_q;
    const double tstar = s.temp1 * s.dth;
    const double qstar = s.temp2 * s.dqh;
    const double forc_th = io.forc_th[c], thv = io.thv[c];
    const double thvstar = tstar * (1.0 + 0.61 * forc_q) + 0.61 * forc_th * qstar;
    double zeta = K.zldis * VKC * GRAV * thvstar / ((ustar * ustar) * thv);
    if (ic::ge0(zeta)) {
        zeta = fmin(P.zetamaxstable, ic::maxc(zeta, 0.01));
        s.um = ic::maxc(K.ur, 0.1);
    } else {
        zeta = ic::ltn(zeta, -0.01) ? zeta : -0.01;
        zeta = ic::gtn(zeta, -100.0) ? zeta : -100.0;
        const double wc = ic::gt0(ustar * thvstar) ? 0.0 : 1.0 * xpow(-GRAV * ustar * thvstar * 1000.0 / thv, 0.333);
        s.um = sqrt(K.ur * K.ur + wc * wc);
    }
    s.zeta = zeta;
    s.obu = K.zldis / zeta;
    if (ic::lt0(s.obuold * s.obu)) s.nmozsgn = s.nmozsgn + 1;
    if (s.nmozsgn >= 4) s.obu = K.zldis / (-0.01);
    s.obuold = s.obu;
    s.itlef = s.itlef + 1;
    if (s.itlef > 2) {
        const double dele = fabs(s.efe - s.efeb);
        s.efeb = s.efe;
        const double det = fmax(s.del, del2);
        s.num_iter = s.itlef;
        if (ic::ltc(det, 0.01) && ic::ltc(dele, 0.1)) return true;
    }
    return s.itlef > A.itmax;
}

// after the iteration (CanopyFluxesMod.F90:1461-1655)
__device__ void finalize(const CanopyArgs& A, const Patch& s, const PatchK& K, double dtime) {
    const ctsmg_canopy_io& io = A.io;
    const int p = s.p, c = s.c, g = s.g;
    const int ldc = io.ldc;
    const int snl = io.snl[c];
    const double frac_sno = io.frac_sno_eff[c], frac_h2osfc = io.frac_h2osfc[c];
    const double ts_top = io.t_soisno[c + (size_t)(snl + NLEVSNO) * ldc];
    const double ts_1 = io.t_soisno[c + (size_t)NLEVSNO * ldc];
    const double lw_grnd = (frac_sno * ipow4(ts_top) + (1.0 - frac_sno - frac_h2osfc) * ipow4(ts_1) +
                            frac_h2osfc * ipow4(io.t_h2osfc[c]));
    const double tb3 = ipow3(s.tlbef);
    const double emv = io.emv[p], emg = io.emg[c];
    io.err_canopy[p] = (1.0 - 0.0) * (io.sabv[p] + K.air + K.bir * tb3 * (s.tlbef + 4.0 * s.dt_veg) + K.cir * lw_grnd) -
                       s.lw_leaf + 0.0 - s.eflx_sh_veg - HVAP * s.qflx_evap_veg - ((s.t_veg - K.tl_ini) * 0.0 / dtime);
    const double thm = io.thm[p], forc_rho = io.forc_rho[c], forc_q = io.forc_q[c];
    const double t_veg = s.t_veg;
    const double delt = s.wtal * io.t_grnd[c] - s.wtl0 * t_veg - s.wta0 * thm - 0.0;
    io.taux[p] = -forc_rho * io.forc_u[g] / s.ram1;
    io.tauy[p] = -forc_rho * io.forc_v[g] / s.ram1;
    io.eflx_sh_grnd[p] = CPAIR * forc_rho * s.wtg * delt;
    io.eflx_sh_snow[p] = CPAIR * forc_rho * s.wtg * (s.wtal * ts_top - s.wtl0 * t_veg - s.wta0 * thm - 0.0);
    io.eflx_sh_soil[p] = CPAIR * forc_rho * s.wtg * (s.wtal * ts_1 - s.wtl0 * t_veg - s.wta0 * thm - 0.0);
    io.eflx_sh_h2osfc[p] = CPAIR * forc_rho * s.wtg * (s.wtal * io.t_h2osfc[c] - s.wtl0 * t_veg - s.wta0 * thm - 0.0);
    io.qflx_evap_soi[p] = forc_rho * s.wtgq * s.delq;
    io.qflx_ev_snow[p] = forc_rho * s.wtgq * (s.wtalq * io.qg_snow[c] - s.wtlq0 * s.qsatl - s.wtaq0 * forc_q);
    io.qflx_ev_soil[p] = forc_rho * s.wtgq * (s.wtalq * io.qg_soil[c] - s.wtlq0 * s.qsatl - s.wtaq0 * forc_q);
    io.qflx_ev_h2osfc[p] = forc_rho * s.wtgq * (s.wtalq * io.qg_h2osfc[c] - s.wtlq0 * s.qsatl - s.wtaq0 * forc_q);
    const double t_ref2m = thm + s.temp1 * s.dth * (1.0 / s.temp12m - 1.0 / s.temp1);
    const double q_ref2m = forc_q + s.temp2 * s.dqh * (1.0 / s.temp22m - 1.0 / s.temp2);
    double qsat_ref2m, e_ref2m;
    qsat(t_ref2m, io.forc_pbot[c], qsat_ref2m, e_ref2m, nullptr);
    const double rh_ref2m = fmin(100.0, q_ref2m / qsat_ref2m * 100.0);
    io.t_ref2m[p] = t_ref2m;
    io.q_ref2m[p] = q_ref2m;
    io.rh_ref2m[p] = rh_ref2m;
    io.vpd_ref2m[p] = e_ref2m * (1.0 - rh_ref2m / 100.0);
    const double forc_lwrad = io.forc_lwrad[c];
    io.dlrad[p] = (1.0 - emv) * emg * forc_lwrad + emv * emg * SB * tb3 * (s.tlbef + 4.0 * s.dt_veg) * (1.0 - 0.0) +
                  emv * emg * SB * 0.0 * (0.0 + 4.0 * 0.0) * 0.0;
    io.ulrad[p] = ((1.0 - emg) * (1.0 - emv) * (1.0 - emv) * forc_lwrad +
                   emv * (1.0 + (1.0 - emg) * (1.0 - emv)) * SB * tb3 * (s.tlbef + 4.0 * s.dt_veg) * (1.0 - 0.0) +
                   emv * (1.0 + (1.0 - emg) * (1.0 - emv)) * SB * 0.0 * (0.0 + 4.0 * 0.0) * 0.0 +
                   emg * (1.0 - emv) * SB * lw_grnd);
    io.t_skin[p] = emv * t_veg + (1.0 - emv) * sqrt(sqrt(lw_grnd));
    const double cgrnds = (A.engine ? 0.0 : io.cgrnds[p]) + CPAIR * forc_rho * s.wtg * s.wtal;
    const double cgrndl = (A.engine ? 0.0 : io.cgrndl[p]) + forc_rho * s.wtgq * s.wtalq * io.dqgdT[c];
    io.cgrnds[p] = cgrnds;
    io.cgrndl[p] = cgrndl;
    io.cgrnd[p] = cgrnds + cgrndl * io.htvp[c];
    double liqcan = K.liqcan, snocan = K.snocan;
    const double snocan_baseline = snocan;
    const double net = (s.qflx_tran_veg - s.qflx_evap_veg) * dtime;
    if (t_veg > TFRZ) {
        if ((s.qflx_evap_veg - s.qflx_tran_veg) * dtime > liqcan) snocan = fmax(0.0, snocan + liqcan + net);
        liqcan = fmax(0.0, liqcan + net);
    } else if (t_veg <= TFRZ) {
        if ((s.qflx_evap_veg - s.qflx_tran_veg) * dtime > snocan) liqcan = liqcan + snocan + net;
        snocan = fmax(0.0, snocan + net);
    }
    if (fabs(snocan) < 1.e-10 * fabs(snocan_baseline)) snocan = 0.0;
    io.liqcan[p] = liqcan;
    io.snocan[p] = snocan;
    if (!A.engine) {
        io.displa[p] = K.displa;
        io.z0mv[p] = K.z0mv;
    }
    io.z0hv[p] = K.z0mv;
    io.z0qv[p] = K.z0mv;
    io.forc_hgt_u_patch[p] = K.hgt_u;
    io.forc_hgt_t_patch[p] = K.hgt_t;
    io.forc_hgt_q_patch[p] = K.hgt_q;
    io.t_veg[p] = t_veg;
    io.taf[p] = s.taf;
    io.qaf[p] = s.qaf;
    io.ustar[p] = s.ustar;
    io.um[p] = s.um;
    io.obu[p] = s.obu;
    io.zeta[p] = s.zeta;
    io.ram1[p] = s.ram1;
    io.rah1[p] = s.rah_a;
    io.raw1[p] = s.raw_a;
    io.rah2[p] = s.rah_b;
    io.raw2[p] = s.rah_b;
    io.rb1[p] = s.rb;
    io.uaf[p] = s.uaf;
    io.rhaf[p] = s.rhaf_last;
    io.vpd[p] = s.vpd_last;
    io.eflx_sh_veg[p] = s.eflx_sh_veg;
    io.qflx_evap_veg[p] = s.qflx_evap_veg;
    io.qflx_tran_veg[p] = s.qflx_tran_veg;
    io.num_iter[p] = s.num_iter;
    io.rssun[p] = s.sun.rs; io.rssha[p] = s.sha.rs;
    io.psnsun[p] = s.sun.psn; io.psnsha[p] = s.sha.psn;
    io.lmrsun[p] = s.sun.lmr; io.lmrsha[p] = s.sha.lmr;
    io.cisun[p] = s.sun.ci; io.cisha[p] = s.sha.ci;
    io.gs_mol_sun[p] = s.sun.gs_mol_phase; io.gs_mol_sha[p] = s.sha.gs_mol_phase;
    io.rh_leaf[p] = s.rh_leaf;
    io.vpd_can[p] = s.vpd_can;
    io.u10_clm[p] = s.u10_clm;
    io.u10[p] = s.u10;
    io.fv[p] = s.ustar;
    io.vds[p] = s.vds;
    io.fm[p] = s.fm;
}

// Work order of the iterating kernel: patches grouped by the branches their
// passes are expected to take -- the surface-layer regime (FrictionVelocity's
// zeta < -zetam, < -zetat, < 0 or stable, from the bulk Richardson number of
// setup), C4 photosynthesis, no PAR in either phase -- so that the lanes of a
// warp mostly follow the same path; in the resident modes the patches that
// needed many passes in the previous step go first, so that long iterations
// do not start at the end of the queue.  Only the schedule changes.
constexpr int NKEY = 64;
struct Order {
    int* key;       // [nfilt] bucket of each filter position
    int* order;     // [nfilt] filter positions in bucket order
    int* hist;      // [NKEY] patches per bucket
    int* fill;      // [NKEY] positions handed out per bucket
};

__device__ __forceinline__ Order order_of(double* ws, int nfilt) {
    int* b = reinterpret_cast<int*>(ws + (size_t)NPD * nfilt) + (size_t)NPI * nfilt;
    return Order{b, b + nfilt, b + 2 * (size_t)nfilt, b + 2 * (size_t)nfilt + NKEY};
}

__global__ void __launch_bounds__(128)
canopy_setup_kernel(CanopyArgs A, int nfilt, const int32_t* __restrict__ filt, double* __restrict__ ws) {
    __shared__ int bh[NKEY];
    if (threadIdx.x < NKEY) bh[threadIdx.x] = 0;
    __syncthreads();
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    const Order O = order_of(ws, nfilt);
    if (f < nfilt) {
        Patch s{};
        PatchK K{};
        Err err{0, 0};
        setup(A, s, K, (filt ? filt[f] : f + A.begp) - A.begp, err);
        s.err_code = err.code;
        s.err_idx = err.idx;
        store_patch(ws, nfilt, f, s);
        store_patchk(ws, nfilt, f, K);
        const double zeta0 = K.zldis / s.obu;
        const bool dark = !(A.io.parsun_z[s.p] > 0.0 || A.io.parsha_z[s.p] > 0.0);
        const int regime = zeta0 < -1.574 ? 3 : zeta0 < -0.465 ? 2 : zeta0 < 0.0 ? 1 : 0;
        int heavy = 2;
        if (A.engine) {
            const int ni = A.io.num_iter[s.p];
            heavy = ni >= 16 ? 0 : ni >= 8 ? 1 : 2;
        }
        const int k = heavy * 16 + regime + (s.c3 ? 0 : 4) + (dark ? 8 : 0);
        O.key[f] = k;
        atomicAdd(&bh[k], 1);
    }
    __syncthreads();
    if (threadIdx.x < NKEY && bh[threadIdx.x]) atomicAdd(&O.hist[threadIdx.x], bh[threadIdx.x]);
}

// Counting-sort scatter of the filter positions by bucket (block-aggregated
// reservations; the order within a bucket is immaterial).
__global__ void __launch_bounds__(128) canopy_order_kernel(int nfilt, double* __restrict__ ws) {
    __shared__ int bh[NKEY], base[NKEY];
    const Order O = order_of(ws, nfilt);
    if (threadIdx.x < NKEY) bh[threadIdx.x] = 0;
    __syncthreads();
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    int k = 0, r = 0;
    if (f < nfilt) {
        k = O.key[f];
        r = atomicAdd(&bh[k], 1);
    }
    __syncthreads();
    if (threadIdx.x < NKEY) {
        int start = 0;
        for (int j = 0; j < (int)threadIdx.x; ++j) start += O.hist[j];
        base[threadIdx.x] = bh[threadIdx.x] ? start + atomicAdd(&O.fill[threadIdx.x], bh[threadIdx.x]) : 0;
    }
    __syncthreads();
    if (f < nfilt) O.order[base[k] + r] = f;
}

#ifndef CTSMG_CANOPY_MIN_BLOCKS
#define CTSMG_CANOPY_MIN_BLOCKS 5
#endif
constexpr int CANOPY_ITERATE_THREADS = 128;
__global__ void __launch_bounds__(CANOPY_ITERATE_THREADS, CTSMG_CANOPY_MIN_BLOCKS)
canopy_iterate_kernel(CanopyArgs A, int nfilt, double* __restrict__ ws, double dtime, int* __restrict__ next) {
    // the lane's PatchK in shared memory (41 doubles a lane: consecutive lanes
    // 82 words apart, so a half-warp's 8-byte accesses hit distinct banks);
    // launched with CANOPY_ITERATE_THREADS threads
    __shared__ PatchK ksh[CANOPY_ITERATE_THREADS];
    PatchK& K = ksh[threadIdx.x];
    Patch s;
    Err err{0, 0};
    const int* __restrict__ order = order_of(ws, nfilt).order;
    int f = -1;                        // filter position of the patch this lane holds
    bool have = true;                  // the work queue was not empty when this lane last looked
    // The loop runs until every lane of the warp is out of work, and the
    // lanes that took a new patch in this iteration meet the others at __syncwarp()
    // before the pass, so each pass is executed by the whole warp at once.
    // (Block size is a multiple of 32 and no lane leaves the loop early.)
#pragma unroll 1
    while (__any_sync(0xffffffffu, have)) {
        if (have && f < 0) {
            const int i = atomicAdd(next, 1);
            if (i >= nfilt) {
                have = false;
            } else {
                f = order[i];
                LANE_PROBE(12);
                load_patch(ws, nfilt, f, s);
                load_patchk(ws, nfilt, f, K);
                err = Err{s.err_code, s.err_idx};
            }
        }
        __syncwarp();
        if (have && pass(A, s, K, err, dtime)) {
            s.err_code = err.code;
            s.err_idx = err.idx;
            store_patch(ws, nfilt, f, s);
            f = -1;
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(128)
canopy_finalize_kernel(CanopyArgs A, int nfilt, const double* __restrict__ ws, double dtime, DevError* derr) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nfilt) return;
    Patch s;
    PatchK K;
    load_patch(ws, nfilt, f, s);
    load_patchk(ws, nfilt, f, K);
    finalize(A, s, K, dtime);
    if (s.err_code) report_error(derr, s.err_idx, 0, s.err_code);
}

} // namespace canopy

// per patch: the record (NPD doubles, NPI ints), its bucket key and its slot
// in the work order; plus the bucket counters
size_t canopy_ws_bytes_per_patch() { return (size_t)canopy::NPD * 8 + (size_t)canopy::NPI * 4 + 8; }

size_t canopy_ws_bytes(int nfilt) {
    return canopy_ws_bytes_per_patch() * (size_t)(nfilt > 0 ? nfilt : 0) + 2 * canopy::NKEY * 4 + 256;
}

cudaError_t launch_canopy(const CanopyArgs& a, int nfilt, const int32_t* d_filt, double dtime, int* d_counter,
                          DevError* err, double* ws, cudaStream_t s) {
    if (nfilt <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    int* counters = reinterpret_cast<int*>(ws + (size_t)canopy::NPD * nfilt) + (size_t)(canopy::NPI + 2) * nfilt;
    e = cudaMemsetAsync(counters, 0, 2 * canopy::NKEY * sizeof(int), s);
    if (e != cudaSuccess) return e;
    const int nb = (nfilt + 127) / 128;
    canopy::canopy_setup_kernel<<<nb, 128, 0, s>>>(a, nfilt, d_filt, ws);
    canopy::canopy_order_kernel<<<nb, 128, 0, s>>>(nfilt, ws);
    int nsm = 152;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    int per_sm = 0;
    // 5 blocks of 41 KB of PatchK per SM: ask for the shared-memory carveout
    cudaFuncSetAttribute(canopy::canopy_iterate_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, canopy::canopy_iterate_kernel,
                                                  canopy::CANOPY_ITERATE_THREADS, 0);
    if (per_sm < 1) per_sm = 1;
    const long long want = (long long)nsm * per_sm;
    const int blocks = (int)(want < nb ? want : nb);
    canopy::canopy_iterate_kernel<<<blocks, canopy::CANOPY_ITERATE_THREADS, 0, s>>>(a, nfilt, ws, dtime, d_counter);
    canopy::canopy_finalize_kernel<<<nb, 128, 0, s>>>(a, nfilt, ws, dtime, err);
    return cudaGetLastError();
}

} // namespace ctsmg

#ifdef CTSMG_LANE_PROBE
extern "C" int32_t ctsmg_lane_probe_read(unsigned long long* out, int32_t reset) {
    cudaError_t e = cudaMemcpyFromSymbol(out, ctsmg::canopy::g_lane_probe, sizeof(unsigned long long) * 64);
    if (reset) {
        unsigned long long z[64] = {};
        cudaMemcpyToSymbol(ctsmg::canopy::g_lane_probe, z, sizeof z);
    }
    return e == cudaSuccess ? 0 : 2;
}
#endif

