// moisture_form_kernels.cu -- SoilWater's moisture form
// (soilwater_movement_method = 1, src/biogeophys/SoilWaterMovementMod.F90:976-1440)
// and the use_flexibleCN negative-liquid fix SoilWater applies after either
// form (:331-368), in FP64 on sm_103a.
//
// The kernels are persistent: a lane owns one column for its whole adaptive
// sub-step loop and, when the column completes, takes the next column of the
// filter, so columns that need many sub-steps do not hold their warp.  A trial
// sub-step streams down the column once: the hydraulic properties of level
// j+1 (compute_hydraulic_properties, :1444-1556, Clapp-Hornberger curve) are
// formed while the flux, its derivatives (compute_moisture_fluxes_and_derivs,
// :1560-1866) and the tridiagonal row of level j (compute_RHS/LHS, :1871-2012)
// are assembled, and each new row is eliminated against the previous one at
// once, in LAPACK dgtsv's order (partial pivoting, NRHS = 1), so only the
// finished U rows, the right-hand side and the per-level values the error
// estimate and the outputs need are kept.  The operation sequence on every
// element is dgtsv's.
#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>
#include <cooperative_groups.h>
#include "ctsm_device.cuh"
#include "soil_math.cuh"
#include "cr_div.cuh"
#include "moisture_form_kernels.cuh"
#include "moisture_form_device.cuh"
#include "hydrology_device.cuh"

namespace ctsmg {

namespace {
constexpr double M_TO_MM = 1.e3;
constexpr int N1 = NLEVSOI + 2;

// std::max / std::min semantics ((a < b) ? b : a), as the oracle evaluates
// them.  Comparisons of the level loop against constants run on the integer
// pipe (fcmp.cuh); these two-variable ones, outside it, stay FP64 compares,
// which need fewer registers than their integer form.
__device__ __forceinline__ double fmx(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double fmn(double a, double b) { return (b < a) ? b : a; }

struct ColView {
    const ctsmg_soilwater_io& io;
    int c, ld;
    __device__ __forceinline__ double ss(const double* b, int j) const { return b[c + (size_t)(j - LS) * ld]; }
    __device__ __forceinline__ double g(const double* b, int j) const { return b[c + (size_t)(j - 1) * ld]; }
    __device__ __forceinline__ double zi(int j) const { return io.zi[c + (size_t)(j + NLEVSNO) * ld]; }
};

// Clapp-Hornberger suction and its derivative w.r.t. volumetric liquid water
// (soil_suction, SoilWaterRetentionCurveClappHornberg1978Mod.F90:95-125; the
// division by watsat is compute_hydraulic_properties' :1540)
// Quotients go through cr_div.cuh (the IEEE quotient's bits but for a/b
// within 2^-79 |a/b| of a rounding midpoint); rws is the level's 1/watsat.
__device__ __forceinline__ void suction(const ColView& k, int j, double s2, const Recip& rws, double& smp,
                                        double& dsmpdw) {
    const double bsw = k.g(k.io.bsw, j);
    smp = -k.g(k.io.sucsat, j) * fm::pow(s2, -bsw);
    const double dsmpds = divf(-bsw * smp, s2);
    dsmpdw = divr(dsmpds, rws);
}

__device__ __forceinline__ double rel_sat(const ColView& k, int j, double liq, const Recip& rws) {
    const double vwc = divf(ic::ltc(liq, 1.0e-6) ? 1.0e-6 : liq, k.ss(k.io.dz, j) * DENH2O);
    double s2 = divr(vwc, rws);
    s2 = ic::gtc(s2, 1.0) ? 1.0 : s2;
    return ic::gtc(s2, 0.01) ? s2 : 0.01;
}
} // namespace

// Per-lane state of one column's adaptive sub-step loop: the persistent
// kernels below run one trial sub-step per loop pass and let a lane whose
// column has completed take the next column, so a column that needs many
// sub-steps does not hold the other lanes of its warp.
// smp_l, hk_l and qout of each trial go straight to the column's arrays (the
// last trial, the one that completes the step, leaves them as the reference
// does), so the lane keeps only its liquid water; the expensive error
// estimate also keeps the flux derivatives.
template <bool EXPENSIVE>
struct MFLane {
    int c, nl, jwt, nsub;
    bool wt;
    double zwt, qinfl, dtsub, dtdone, qcharge, vwc_q, imped_q;
    double liq[N1];
    double dqodw1[EXPENSIVE ? N1 : 1], dqodw2[EXPENSIVE ? N1 : 1];
};

enum { MF_MORE = 0, MF_DONE = 1, MF_SINGULAR = 2, MF_NOT_DONE = 3 };

template <bool EXPENSIVE>
__device__ __forceinline__ void mf_begin(MFLane<EXPENSIVE>& L, const ctsmg_soilwater_io& io, int c, const MoistureFormArgs& P) {
    const ColView k{io, c, io.ldc};
    L.c = c;
    L.nl = io.nbedrock[c];
    L.qinfl = io.qflx_infl[c];
    L.zwt = io.zwt[c];
    L.wt = P.lower_bc == 3;
    L.jwt = NLEVSOI;
    if (L.wt) {
#pragma unroll 1
        for (int j = 1; j <= NLEVSOI; ++j)
            if (ic::le(L.zwt, k.zi(j))) { L.jwt = j - 1; break; }
    }
#pragma unroll 1
    for (int j = 1; j <= L.nl; ++j) L.liq[j] = k.ss(io.h2osoi_liq, j);
    L.nsub = 0;
    L.dtsub = P.dtime;
    L.dtdone = 0.0;
    L.qcharge = 0.0;
    L.vwc_q = 0.0;
    L.imped_q = 1.0;
}

// One trial sub-step (SoilWaterMovementMod.F90:1197-1399).  Returns MF_MORE,
// MF_DONE, MF_SINGULAR (with *info = dgtsv's info) or MF_NOT_DONE when the
// loop has run P.max_trials trials (a bound the reference's halving /
// doubling rule cannot reach).
template <bool EXPENSIVE>
__device__ int mf_trial(MFLane<EXPENSIVE>& L, const ctsmg_soilwater_io& io, const MoistureFormArgs& P, int* info) {
    const ColView k{io, L.c, io.ldc};
    const int nl = L.nl, jwt = L.jwt;
    const bool wt = L.wt;
    const size_t ld = io.ldc;
    double* const qout_c = io.qout + L.c;     // level j at qout_c[(j-1) ld]
    double d[N1], du[N1], dl2[N1], b[N1];
    L.nsub = L.nsub + 1;
    const double dtsub = L.dtsub;
    // ---- level 1 suction, then stream the levels
    Recip rws_c = recip(k.g(io.watsat, 1));
    double s2c = rel_sat(k, 1, L.liq[1], rws_c);
    double smp_c, dsmpdw_c;
    suction(k, 1, s2c, rws_c, smp_c, dsmpdw_c);
    double qin = L.qinfl, dqidw0 = 0.0, dqidw1 = 0.0;
    double hk_nl = 0.0, dhkdw_nl = 0.0, qo_nl = 0.0, dq1_nl = 0.0;
    // pending dgtsv row: d_p, du_p, b_p; its sub-diagonal arrives with the next row
    double d_p = 0.0, du_p = 0.0, b_p = 0.0;
#pragma unroll 1
    for (int j = 1; j <= nl; ++j) {
        double s2n = 0.0, smp_n = 0.0, dsmpdw_n = 0.0;
        Recip rws_n = rws_c;
        if (j < nl) {
            rws_n = recip(k.g(io.watsat, j + 1));
            s2n = rel_sat(k, j + 1, L.liq[j + 1], rws_n);
            suction(k, j + 1, s2n, rws_n, smp_n, dsmpdw_n);
        }
        double s1, imped;
        if (j == nl) {
            s1 = s2c;
            imped = pow10_dd(-P.e_ice * k.g(io.icefrac, j));
        } else {
            s1 = 0.5 * (s2c + s2n);
            imped = pow10_dd(-P.e_ice * (0.5 * (k.g(io.icefrac, j) + k.g(io.icefrac, j + 1))));
        }
        s1 = ic::gtc(s1, 1.0) ? 1.0 : s1;
        s1 = ic::gtc(s1, 0.01) ? s1 : 0.01;
        const double bsw = k.g(io.bsw, j);
        const double hkj = imped * k.g(io.hksat, j) * fm::pow(s1, 2.0 * bsw + 3.0);
        const double dhkdw = divf((2.0 * bsw + 3.0) * hkj, s1);
        io.smp_l[L.c + (j - 1) * ld] = smp_c;
        io.hk_l[L.c + (j - 1) * ld] = hkj;
        if (wt && j == jwt + 1) {
            L.vwc_q = divf(ic::ltc(L.liq[j], 1.0e-6) ? 1.0e-6 : L.liq[j], k.ss(io.dz, j) * DENH2O);
            L.imped_q = imped;
        }
        // flux out of the bottom of level j and its derivatives
        double qo, dq1, dq2;
        if (j < nl) {
            const double dhkds1 = divr(0.5 * dhkdw, rws_c);
            const double dhkds2 = divr(0.5 * dhkdw, rws_n);
            const double num = smp_n - smp_c;
            const Recip rden = recip(M_TO_MM * (k.ss(io.z, j + 1) - k.ss(io.z, j)));
            qo = divr(-hkj * num, rden) + hkj;
            dq1 = divr(hkj * dsmpdw_c - dhkds1 * num, rden) + dhkds1;
            dq2 = divr(-hkj * dsmpdw_n - dhkds2 * num, rden) + dhkds2;
        } else if (P.lower_bc == 3) {            // bc_waterTable (nl == nlevsoi)
            if (NLEVSOI > jwt) {
                qo = 0.0; dq1 = 0.0; dq2 = 0.0;
            } else {
                const double dhkds1 = divr(dhkdw, rws_c);
                const double num = -smp_c;
                const Recip rden = recip(M_TO_MM * (L.zwt - k.ss(io.z, j)));
                qo = divr(-hkj * num, rden) + hkj;
                dq1 = divr(hkj * dsmpdw_c - dhkds1 * num, rden) + dhkds1;
                dq2 = 0.0;
            }
        } else if (P.lower_bc == 1) {            // bc_flux: free drainage
            qo = hkj; dq1 = divr(dhkdw, rws_c); dq2 = 0.0;
        } else {                                 // bc_zero_flux
            qo = 0.0; dq1 = 0.0; dq2 = 0.0;
        }
        qout_c[(j - 1) * ld] = qo;
        if (EXPENSIVE) { L.dqodw1[j] = dq1; L.dqodw2[j] = dq2; }
        if (j == nl) { hk_nl = hkj; dhkdw_nl = dhkdw; qo_nl = qo; dq1_nl = dq1; }
        // tridiagonal row j
        const double dt_dz = divf(dtsub, M_TO_MM * k.ss(io.dz, j));
        const double amx = (j == 1) ? 0.0 : dqidw0 * dt_dz;
        const double bmx = -1.0 - (-dqidw1 + dq1) * dt_dz;
        const double cmx = (j == nl) ? 0.0 : -dq2 * dt_dz;
        const double fluxNet = qin - qo - k.g(io.qflx_rootsoi, j);
        const double rmx = -fluxNet * dt_dz;
        if (j == 1) {
            d_p = bmx; du_p = cmx; b_p = rmx;
        } else {
            // dgtsv elimination step i = j-2 (0-based) on rows j-1 (pending) and j
            double dl = amx, dn = bmx, dun = cmx, bn = rmx;
            if (ic::abs_ge(d_p, dl)) {
                if (!ic::ne0(d_p)) { *info = j - 1; return MF_SINGULAR; }
                const double fact = divf(dl, d_p);
                dn = dn - fact * du_p;
                bn = bn - fact * b_p;
                dl2[j - 1] = 0.0;
            } else {
                const double fact = divf(d_p, dl);
                d_p = dl;
                const double temp = dn;
                dn = du_p - fact * temp;
                dl2[j - 1] = dun;                 // second super-diagonal fill of row j-1
                dun = -fact * dun;
                du_p = temp;
                const double tb = b_p;
                b_p = bn;
                bn = tb - fact * bn;
            }
            d[j - 1] = d_p; du[j - 1] = du_p; b[j - 1] = b_p;
            d_p = dn; du_p = dun; b_p = bn;
        }
        // next level
        qin = qo; dqidw0 = dq1; dqidw1 = dq2;
        s2c = s2n; smp_c = smp_n; dsmpdw_c = dsmpdw_n; rws_c = rws_n;
    }
    if (!ic::ne0(d_p)) { *info = nl; return MF_SINGULAR; }
    d[nl] = d_p; du[nl] = du_p; b[nl] = b_p;
    // back substitution (1-based rows here)
    b[nl] = divf(b[nl], d[nl]);
    if (nl > 1) b[nl - 1] = divf(b[nl - 1] - du[nl - 1] * b[nl], d[nl - 1]);
#pragma unroll 1
    for (int i = nl - 2; i >= 1; --i) b[i] = divf(b[i] - du[i] * b[i + 1] - dl2[i] * b[i + 2], d[i]);
    // ---- error estimate (:1306-1348)
    double errorMax = 0.0;
#pragma unroll 1
    for (int j = 1; j <= nl; ++j) {
        const double dt_dz = divf(dtsub, M_TO_MM * k.ss(io.dz, j));
        const double qi = (j == 1) ? L.qinfl : qout_c[(j - 2) * ld];
        const double qo = qout_c[(j - 1) * ld];
        double fluxNet0;
        if (EXPENSIVE) {
            const double qin_test = (j == 1) ? qi + 0.0 * b[j]
                                             : qi + L.dqodw1[j - 1] * b[j - 1] + L.dqodw2[j - 1] * b[j];
            const double qout_test = (j == nl) ? qo + L.dqodw1[j] * b[j]
                                               : qo + L.dqodw1[j] * b[j] + L.dqodw2[j] * b[j + 1];
            fluxNet0 = qin_test - qout_test - k.g(io.qflx_rootsoi, j);
        } else {
            fluxNet0 = divf(b[j], dt_dz);
        }
        // fluxNet1, the net flux at the start of the sub-step, as the row's rmx had it
        const double fn1 = qi - qo - k.g(io.qflx_rootsoi, j);
        const double e = fabs(fn1 - fluxNet0) * dtsub * 0.5;
        errorMax = (j == 1) ? e : ((errorMax < e) ? e : errorMax);
    }
    if (errorMax > P.xTolerUpper && dtsub > P.dtmin) {
        L.dtsub = fmx(dtsub / 2.0, P.dtmin);
        return (L.nsub >= P.max_trials) ? MF_NOT_DONE : MF_MORE;
    }
#pragma unroll 1
    for (int j = 1; j <= nl; ++j) L.liq[j] = L.liq[j] + b[j] * (M_TO_MM * k.ss(io.dz, j));
    double qcTemp;
    if (P.lower_bc == 1) qcTemp = hk_nl + dhkdw_nl * b[nl];
    else if (P.lower_bc == 2) qcTemp = 0.0;
    else qcTemp = qo_nl + dq1_nl * b[nl];
    L.qcharge = L.qcharge + qcTemp * (dtsub / P.dtime);
    L.dtdone = L.dtdone + dtsub;
    if (fabs(P.dtime - L.dtdone) < P.verySmall) return MF_DONE;
    double nd = dtsub;
    if (errorMax < P.xTolerLower) nd = nd * 2.0;
    L.dtsub = fmn(nd, P.dtime - L.dtdone);
    return (L.nsub >= P.max_trials) ? MF_NOT_DONE : MF_MORE;
}

// The end of soilwater_moisture_form for a completed column (:1401-1436).
template <bool EXPENSIVE>
__device__ void mf_finish(MFLane<EXPENSIVE>& L, const ctsmg_soilwater_io& io, const MoistureFormArgs& P) {
    const ColView k{io, L.c, io.ldc};
    const int c = L.c, nl = L.nl, jwt = L.jwt;
    io.num_substeps[c] = (double)L.nsub;
    // over-saturated layers pass their excess upward (:1405-1409)
#pragma unroll 1
    for (int j = nl; j >= 2; --j) {
        const double cap = k.g(io.eff_porosity, j) * M_TO_MM * k.ss(io.dz, j);
        const double over = ic::lt0(L.liq[j] - cap) ? 0.0 : L.liq[j] - cap;
        L.liq[j] = fmn(cap, L.liq[j]);
        L.liq[j - 1] = L.liq[j - 1] + over;
    }
    double* h2osoi_liq = io.h2osoi_liq;
#pragma unroll 1
    for (int j = 1; j <= nl; ++j) {
        h2osoi_liq[c + (size_t)(j - LS) * k.ld] = L.liq[j];
        io.qin[c + (size_t)(j - 1) * k.ld] = (j == 1) ? L.qinfl : io.qout[c + (size_t)(j - 2) * k.ld];
    }
    double qcharge = L.qcharge;
    // compute_qcharge for the water-table boundary (:2016-2135)
    if (L.wt && jwt < NLEVSOI) {
        const double zwt = L.zwt;
        const double wh_zwt = -k.g(io.sucsat, jwt + 1) - zwt * M_TO_MM;
        double s1 = L.vwc_q / k.g(io.watsat, jwt + 1);
        s1 = ic::ltc(s1, 0.01) ? 0.01 : s1;
        s1 = ic::ltc(s1, 1.0) ? s1 : 1.0;
        const double ka = L.imped_q * k.g(io.hksat, jwt + 1) * fm::pow(s1, 2.0 * k.g(io.bsw, jwt + 1) + 3.0);
        const int jm = jwt > 1 ? jwt : 1;
        const double smp1 = fmx(io.smpmin[c], io.smp_l[c + (size_t)(jm - 1) * k.ld]);
        const double wh = smp1 - k.ss(io.z, jm) * M_TO_MM;
        if (jwt == 0) qcharge = -ka * (wh_zwt - wh) / ((zwt + (double)1.e-3f) * M_TO_MM);
        else qcharge = -ka * (wh_zwt - wh) / ((zwt - k.ss(io.z, jwt)) * M_TO_MM * 2.0);
        qcharge = fmx(-10.0 / P.dtime, qcharge);
        qcharge = fmn(10.0 / P.dtime, qcharge);
    }
    io.qcharge[c] = qcharge;
}

// The next filter position for the calling lane: the lanes that ask at the
// same time take consecutive positions with one atomic, so a warp's first
// columns (and most refills) are neighbours in memory.
__device__ __forceinline__ int mf_grab(int* counter) {
    namespace cg = cooperative_groups;
    cg::coalesced_group g = cg::coalesced_threads();
    int base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(counter, (int)g.size());
    base = g.shfl(base, 0);
    return base + (int)g.thread_rank();
}

// The persistent loop: begin(fc) prepares filter position fc and returns its
// column; end(fc, status, info) finishes it.
template <bool EXPENSIVE, class Begin, class End>
__device__ __forceinline__ void mf_persistent(const ctsmg_soilwater_io& io, int n, int* counter,
                                              const MoistureFormArgs& P, Begin begin, End end) {
    MFLane<EXPENSIVE> L;
    int fc = mf_grab(counter);
    if (fc >= n) return;
    mf_begin(L, io, begin(fc), P);
#pragma unroll 1
    for (;;) {
        int info = 0;
        const int st = mf_trial(L, io, P, &info);
        if (st == MF_MORE) continue;
        if (st == MF_DONE) mf_finish(L, io, P);
        end(fc, L.c, st, info);
        fc = mf_grab(counter);
        if (fc >= n) break;
        mf_begin(L, io, begin(fc), P);
    }
}

template <bool EXPENSIVE>
__global__ void __launch_bounds__(128)
moisture_form_kernel(ctsmg_soilwater_io io, int begc, int nfilt, const int32_t* __restrict__ filt,
                     MoistureFormArgs P, DevError* err, int* counter) {
    mf_persistent<EXPENSIVE>(io, nfilt, counter, P,
                  [&](int fc) { return (filt ? filt[fc] : fc + begc) - begc; },
                  [&](int fc, int c, int st, int info) {
                      if (st == MF_SINGULAR) report_error(err, c + begc, info, CTSMG_E_SINGULAR);
                      else if (st == MF_NOT_DONE) report_error(err, c + begc, 0, CTSMG_E_TIMEOUT);
                  });
}

__global__ void __launch_bounds__(128)
flexcn_kernel(ctsmg_soilwater_io io, int begc, int nfilt, const int32_t* __restrict__ filt) {
    const int fc = blockIdx.x * blockDim.x + threadIdx.x;
    if (fc >= nfilt) return;
    flexcn_column(io, (filt ? filt[fc] : fc + begc) - begc);
}

// One column's soil-water part of a resident model step with the moisture
// form: SetSoilWaterFractions, SoilWater (moisture form), the flexibleCN fix
// and, if refresh, the between-step h2osoi_vol refresh
// (HydrologyNoDrainageMod.F90:302, 346, 580, 590).
// The resident step's moisture-form SoilWater in three launches, so that the
// persistent sub-step kernel holds nothing but the sub-step loop and its
// lanes stay converged outside it: before it, one thread per column runs
// SetSoilWaterFractions (and with HYDRO SaturatedExcessRunoff and the
// infiltration chain that yields qflx_infl); after it, the flexibleCN fix,
// with HYDRO the water tables and lateral flows, and the h2osoi_vol refresh.
__device__ __forceinline__ ctsmg_soilhydrology_params column_params(const HydroStepArgs& hy, int c) {
    ctsmg_soilhydrology_params hp = hy.par;
    if (hy.baseflow_scalar_c) hp.baseflow_scalar = hy.baseflow_scalar_c[c];
    if (hy.fff_c) hp.fff = hy.fff_c[c];
    return hp;
}

struct MfOrder {
    int* hist;      // [MF_NKEY] positions per bucket
    int* fill;      // [MF_NKEY] positions handed out per bucket
    int* key;       // [ncol] bucket of each position
    int* order;     // [ncol] positions in bucket order
};

__host__ __device__ __forceinline__ MfOrder mf_order_of(int* w, int ncol) {
    return MfOrder{w + 32, w + 32 + MF_NKEY, w + MF_WORK_HEAD, w + MF_WORK_HEAD + ncol};
}

// Bucket of a column: sub-step class of the previous step (a count that is
// not a number, or 0 before the first step, counts as 1), then bedrock depth,
// both descending.
__device__ __forceinline__ int mf_key(double nsub_prev, int nl) {
    int cls = 0;
    if (nsub_prev > 1.5) cls = 1;
    if (nsub_prev > 2.5) cls = 2;
    if (nsub_prev > 4.5) cls = 3;
    if (nsub_prev > 8.5) cls = 4;
    if (nsub_prev > 16.5) cls = 5;
    nl = nl < 1 ? 1 : (nl > NLEVSOI ? NLEVSOI : nl);
    return (MF_NCLS - 1 - cls) * NLEVSOI + (NLEVSOI - nl);
}

template <bool HYDRO, bool SORT>
__global__ void __launch_bounds__(128)
mf_pre_kernel(ctsmg_soilwater_io io, int ncol, double dtime, const int32_t* __restrict__ filt, HydroStepArgs hy,
              int* work) {
    __shared__ int bh[SORT ? MF_NKEY : 1];
    if (SORT) {
        for (int i = threadIdx.x; i < MF_NKEY; i += blockDim.x) bh[i] = 0;
        __syncthreads();
    }
    const int fc = blockIdx.x * blockDim.x + threadIdx.x;
    if (fc < ncol) {
        const int c = filt ? filt[fc] - 1 : fc;
        set_soil_water_fractions(io, c);
        if (HYDRO) {
            const ctsmg_soilhydrology_params hp = column_params(hy, c);
            hydro::saturated_excess_runoff(hy.io, c, hp.fff);
            hydro::infiltration_chain(hy.io, c, hp, dtime);
        }
        if (SORT) {
            const int k = mf_key(io.num_substeps[c], io.nbedrock[c]);
            mf_order_of(work, ncol).key[fc] = k;
            atomicAdd(&bh[k], 1);
        }
    }
    if (SORT) {
        __syncthreads();
        int* hist = mf_order_of(work, ncol).hist;
        for (int i = threadIdx.x; i < MF_NKEY; i += blockDim.x)
            if (bh[i]) atomicAdd(&hist[i], bh[i]);
    }
}

// Scatter of the filter positions into bucket order: a block ranks its own
// positions within each bucket in shared memory and takes one run of slots
// per bucket from the bucket's fill counter.  (The order within a bucket
// depends on block timing; every column's result is independent of it.)
__global__ void __launch_bounds__(128) mf_order_kernel(int ncol, int* work) {
    __shared__ int bh[MF_NKEY], start[MF_NKEY];
    const MfOrder O = mf_order_of(work, ncol);
    for (int i = threadIdx.x; i < MF_NKEY; i += blockDim.x) bh[i] = 0;
    if (threadIdx.x < 32) {             // exclusive prefix sum of the histogram by warp 0
        constexpr int PER = (MF_NKEY + 31) / 32;
        const int lane = threadIdx.x;
        int v[PER], sum = 0;
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int i = lane * PER + q;
            v[q] = i < MF_NKEY ? O.hist[i] : 0;
            sum += v[q];
        }
        int inc = sum;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, inc, off);
            if (lane >= off) inc += t;
        }
        int run = inc - sum;
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int i = lane * PER + q;
            if (i < MF_NKEY) start[i] = run;
            run += v[q];
        }
    }
    __syncthreads();
    const int fc = blockIdx.x * blockDim.x + threadIdx.x;
    int k = 0, r = 0;
    if (fc < ncol) {
        k = O.key[fc];
        r = atomicAdd(&bh[k], 1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < MF_NKEY; i += blockDim.x)
        if (bh[i]) start[i] += atomicAdd(&O.fill[i], bh[i]);
    __syncthreads();
    if (fc < ncol) O.order[start[k] + r] = fc;
}

#ifndef CTSMG_MF_MIN_BLOCKS
#define CTSMG_MF_MIN_BLOCKS 1
#endif
template <bool EXPENSIVE>
__global__ void __launch_bounds__(128, CTSMG_MF_MIN_BLOCKS)
mf_core_kernel(ctsmg_soilwater_io io, int ncol, MoistureFormArgs P, DevError* err, const int32_t* __restrict__ filt,
               int* counter, const int* __restrict__ order, int compact) {
    // compact: io holds the columns of the work order at positions 0..ncol-1
    // (order maps a position back to its filter position, for errors)
    mf_persistent<EXPENSIVE>(io, ncol, counter, P,
                  [&](int fc) {
                      if (compact) return fc;
                      const int p = order ? order[fc] : fc;
                      return filt ? filt[p] - 1 : p;
                  },
                  [&](int fc, int c, int st, int info) {
                      int col = c;
                      if (compact) {
                          const int q = order[c];
                          col = filt ? filt[q] - 1 : q;
                      }
                      if (st == MF_SINGULAR) report_error(err, col + 1, info, CTSMG_E_SINGULAR);
                      else if (st == MF_NOT_DONE) report_error(err, col + 1, 0, CTSMG_E_TIMEOUT);
                  });
}

// Compact mode: the components the sub-step kernel reads and writes, moved
// for the columns of the work order into a workspace in that order (a warp's
// columns then sit side by side in memory and run level loops of one length),
// and the written ones moved back afterwards.  Each move copies rows
// [row0, row0 + rows) of one component; the workspace arrays have the
// component's own row layout with the work order's length as leading
// dimension, so the kernel's indexing is unchanged.
struct MfMove {
    char* orig;             // the component (the step's leading dimension)
    char* work;             // its workspace copy (leading dimension ncol)
    int row0, rows, esize, out;
};
struct MfMoves {
    MfMove m[MF_MOVES];
    int n;
};

__global__ void __launch_bounds__(128)
mf_move_kernel(MfMoves mv, int n, int ld, const int* __restrict__ order, const int32_t* __restrict__ filt, int back) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int q = order[p];
    const int c = filt ? filt[q] - 1 : q;
    for (int i = 0; i < mv.n; ++i) {
        const MfMove& M = mv.m[i];
        if (back && !M.out) continue;
        for (int r = M.row0; r < M.row0 + M.rows; ++r) {
            const size_t o = (size_t)r * ld + c, w = (size_t)r * n + p;
            if (M.esize == 8) {
                double* a = reinterpret_cast<double*>(M.orig);
                double* b = reinterpret_cast<double*>(M.work);
                if (back) a[o] = b[w];
                else b[w] = a[o];
            } else {
                int32_t* a = reinterpret_cast<int32_t*>(M.orig);
                int32_t* b = reinterpret_cast<int32_t*>(M.work);
                if (back) a[o] = b[w];
                else b[w] = a[o];
            }
        }
    }
}

namespace {
// The moves of compact mode and the workspace io (pointers into `ws`, which
// holds mf_compact_bytes(ncol) bytes): sets cio and mv, returns the bytes used.
size_t mf_compact_layout(const ctsmg_soilwater_io& io, int ncol, char* ws, ctsmg_soilwater_io* cio, MfMoves* mv) {
    constexpr int SS = NLEVSNO + NLEVGRND, ZI = NLEVSNO + NLEVGRND + 1;
    *cio = io;
    cio->ldc = ncol;
    mv->n = 0;
    size_t off = 0;
    auto add = [&](auto*& dptr, auto* optr, int kind_rows, int row0, int rows, int esize, int out) {
        char* w = ws ? ws + off : nullptr;
        off += ((size_t)kind_rows * ncol * esize + 255) / 256 * 256;
        if (!ws) return;
        MfMove& M = mv->m[mv->n++];
        M.orig = reinterpret_cast<char*>(const_cast<void*>(static_cast<const void*>(optr)));
        M.work = w;
        M.row0 = row0;
        M.rows = rows;
        M.esize = esize;
        M.out = out;
        using T = std::remove_reference_t<decltype(dptr)>;
        dptr = reinterpret_cast<T>(w);
    };
    // levels 1..nlevsoi of the snow+soil and interface components
    add(cio->z, io.z, SS, NLEVSNO, NLEVSOI, 8, 0);
    add(cio->dz, io.dz, SS, NLEVSNO, NLEVSOI, 8, 0);
    add(cio->h2osoi_liq, io.h2osoi_liq, SS, NLEVSNO, NLEVSOI, 8, 1);
    add(cio->zi, io.zi, ZI, NLEVSNO, NLEVSOI + 1, 8, 0);
    add(cio->watsat, io.watsat, NLEVGRND, 0, NLEVSOI, 8, 0);
    add(cio->sucsat, io.sucsat, NLEVGRND, 0, NLEVSOI, 8, 0);
    add(cio->bsw, io.bsw, NLEVGRND, 0, NLEVSOI, 8, 0);
    add(cio->hksat, io.hksat, NLEVGRND, 0, NLEVSOI, 8, 0);
    add(cio->eff_porosity, io.eff_porosity, NLEVGRND, 0, NLEVSOI, 8, 0);
    add(cio->icefrac, io.icefrac, NLEVGRND, 0, NLEVSOI, 8, 0);
    add(cio->smp_l, io.smp_l, NLEVGRND, 0, NLEVSOI, 8, 1);
    add(cio->hk_l, io.hk_l, NLEVGRND, 0, NLEVSOI, 8, 1);
    add(cio->qflx_rootsoi, io.qflx_rootsoi, NLEVSOI, 0, NLEVSOI, 8, 0);
    add(cio->qin, io.qin, NLEVSOI, 0, NLEVSOI, 8, 1);
    add(cio->qout, io.qout, NLEVSOI, 0, NLEVSOI, 8, 1);
    add(cio->zwt, io.zwt, 1, 0, 1, 8, 0);
    add(cio->smpmin, io.smpmin, 1, 0, 1, 8, 0);
    add(cio->qflx_infl, io.qflx_infl, 1, 0, 1, 8, 0);
    add(cio->qcharge, io.qcharge, 1, 0, 1, 8, 1);
    add(cio->num_substeps, io.num_substeps, 1, 0, 1, 8, 1);
    add(cio->nbedrock, io.nbedrock, 1, 0, 1, 4, 0);
    return off;
}
} // namespace

size_t mf_compact_bytes(int ncol) {
    ctsmg_soilwater_io io{}, cio{};
    MfMoves mv;
    return mf_compact_layout(io, ncol > 0 ? ncol : 0, nullptr, &cio, &mv);
}

template <bool HYDRO>
__global__ void __launch_bounds__(128)
mf_post_kernel(ctsmg_soilwater_io io, int ncol, double dtime, int flexcn, int refresh,
               const int32_t* __restrict__ filt, HydroStepArgs hy) {
    const int fc = blockIdx.x * blockDim.x + threadIdx.x;
    if (fc >= ncol) return;
    const int c = filt ? filt[fc] - 1 : fc;
    if (flexcn) flexcn_column(io, c);
    if (HYDRO) {
        const ctsmg_soilhydrology_params hp = column_params(hy, c);
        hydro::perched_water_table(hy.io, c);
        hydro::theta_based_water_table(hy.io, c);
        hydro::perched_lateral_flow(hy.io, c, hp, dtime);
        hydro::subsurface_lateral_flow(hy.io, c, hp, dtime);
    }
    if (refresh) refresh_h2osoi_vol(io, c);
}

// Blocks of a persistent launch: every SM filled to the kernel's occupancy.
template <class K>
static int persistent_blocks(K kernel, int n) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, 0);
    const int full = (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
    const int need = (n + 127) / 128;
    return need < full ? need : full;
}

cudaError_t launch_mf_step(const ctsmg_soilwater_io& io, int ncol, const MoistureFormArgs& P, int flexcn, int refresh,
                           DevError* err, const int32_t* d_filt, cudaStream_t s, int* d_work,
                           const HydroStepArgs* hy, bool sorted, void* d_compact) {
    if (ncol <= 0) return cudaSuccess;
    const int nb = (ncol + 127) / 128;
    const HydroStepArgs none{};
    cudaError_t e = cudaMemsetAsync(d_work, 0, (sorted ? MF_WORK_HEAD : 1) * sizeof(int), s);
    if (e != cudaSuccess) return e;
    const HydroStepArgs& ha = hy ? *hy : none;
    if (hy && sorted) mf_pre_kernel<true, true><<<nb, 128, 0, s>>>(io, ncol, P.dtime, d_filt, ha, d_work);
    else if (hy) mf_pre_kernel<true, false><<<nb, 128, 0, s>>>(io, ncol, P.dtime, d_filt, ha, d_work);
    else if (sorted) mf_pre_kernel<false, true><<<nb, 128, 0, s>>>(io, ncol, P.dtime, d_filt, ha, d_work);
    else mf_pre_kernel<false, false><<<nb, 128, 0, s>>>(io, ncol, P.dtime, d_filt, ha, d_work);
    const int* order = nullptr;
    const bool compact = sorted && d_compact;
    ctsmg_soilwater_io cio = io;
    MfMoves mv;
    mv.n = 0;
    if (sorted) {
        mf_order_kernel<<<nb, 128, 0, s>>>(ncol, d_work);
        order = mf_order_of(d_work, ncol).order;
    }
    if (compact) {
        mf_compact_layout(io, ncol, static_cast<char*>(d_compact), &cio, &mv);
        mf_move_kernel<<<nb, 128, 0, s>>>(mv, ncol, io.ldc, order, d_filt, 0);
    }
    if (P.expensive)
        mf_core_kernel<true><<<persistent_blocks(mf_core_kernel<true>, ncol), 128, 0, s>>>(
            cio, ncol, P, err, d_filt, d_work, order, compact ? 1 : 0);
    else
        mf_core_kernel<false><<<persistent_blocks(mf_core_kernel<false>, ncol), 128, 0, s>>>(
            cio, ncol, P, err, d_filt, d_work, order, compact ? 1 : 0);
    if (compact) mf_move_kernel<<<nb, 128, 0, s>>>(mv, ncol, io.ldc, order, d_filt, 1);
    if (hy) mf_post_kernel<true><<<nb, 128, 0, s>>>(io, ncol, P.dtime, flexcn, refresh, d_filt, *hy);
    else if (flexcn || refresh) mf_post_kernel<false><<<nb, 128, 0, s>>>(io, ncol, P.dtime, flexcn, refresh, d_filt, none);
    return cudaGetLastError();
}

cudaError_t launch_moisture_form(const ctsmg_soilwater_io& io, int begc, int nfilt, const int32_t* d_filt,
                                 const MoistureFormArgs& P, DevError* err, cudaStream_t s, int* d_counter) {
    if (nfilt <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    if (P.expensive)
        moisture_form_kernel<true><<<persistent_blocks(moisture_form_kernel<true>, nfilt), 128, 0, s>>>(
            io, begc, nfilt, d_filt, P, err, d_counter);
    else
        moisture_form_kernel<false><<<persistent_blocks(moisture_form_kernel<false>, nfilt), 128, 0, s>>>(
            io, begc, nfilt, d_filt, P, err, d_counter);
    return cudaGetLastError();
}

// SetSoilWaterFractions (src/biogeophys/SoilHydrologyMod.F90:236-249) as a
// drop-in over a column filter.
__global__ void __launch_bounds__(128)
swfrac_kernel(ctsmg_soilwater_io io, int begc, int nfilt, const int32_t* __restrict__ filt) {
    const int fc = blockIdx.x * blockDim.x + threadIdx.x;
    if (fc >= nfilt) return;
    set_soil_water_fractions(io, (filt ? filt[fc] : fc + begc) - begc);
}

cudaError_t launch_set_soil_water_fractions(const ctsmg_soilwater_io& io, int begc, int nfilt, const int32_t* d_filt,
                                            cudaStream_t s) {
    if (nfilt <= 0) return cudaSuccess;
    swfrac_kernel<<<(nfilt + 127) / 128, 128, 0, s>>>(io, begc, nfilt, d_filt);
    return cudaGetLastError();
}

cudaError_t launch_flexcn(const ctsmg_soilwater_io& io, int begc, int nfilt, const int32_t* d_filt, cudaStream_t s) {
    if (nfilt <= 0) return cudaSuccess;
    flexcn_kernel<<<(nfilt + 127) / 128, 128, 0, s>>>(io, begc, nfilt, d_filt);
    return cudaGetLastError();
}

} // namespace ctsmg
