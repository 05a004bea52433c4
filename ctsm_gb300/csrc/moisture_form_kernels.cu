// moisture_form_kernels.cu -- SoilWater's moisture form
// (soilwater_movement_method = 1, src/biogeophys/SoilWaterMovementMod.F90:976-1440)
// and the use_flexibleCN negative-liquid fix SoilWater applies after either
// form (:331-368), in FP64 on sm_103a.
//
// One thread owns one column for the whole adaptive sub-step loop.  A trial
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
#include "ctsm_device.cuh"
#include "soil_math.cuh"
#include "moisture_form_kernels.cuh"
#include "moisture_form_device.cuh"
#include "hydrology_device.cuh"

namespace ctsmg {

namespace {
constexpr double M_TO_MM = 1.e3;
constexpr int N1 = NLEVSOI + 2;

// std::max / std::min semantics ((a < b) ? b : a), as the oracle evaluates them
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
__device__ __forceinline__ void suction(const ColView& k, int j, double s2, double& smp, double& dsmpdw) {
    const double bsw = k.g(k.io.bsw, j);
    smp = -k.g(k.io.sucsat, j) * pow(s2, -bsw);
    const double dsmpds = -bsw * smp / s2;
    dsmpdw = dsmpds / k.g(k.io.watsat, j);
}

__device__ __forceinline__ double rel_sat(const ColView& k, int j, double liq) {
    const double vwc = fmx(liq, 1.0e-6) / (k.ss(k.io.dz, j) * DENH2O);
    double s2 = vwc / k.g(k.io.watsat, j);
    s2 = fmn(s2, 1.0);
    return fmx(0.01, s2);
}
} // namespace

// Returns 0, dgtsv's info (1-based level of the zero pivot), or -1 when the
// sub-step loop has not completed the step within P.max_trials trials (the
// host sets a bound the reference's halving/doubling rule cannot reach).
__device__ int mf_column(const ctsmg_soilwater_io& io, int c, const MoistureFormArgs& P) {
    const ColView k{io, c, io.ldc};
    const int nl = io.nbedrock[c];
    const double qinfl = io.qflx_infl[c];
    const double zwt = io.zwt[c];
    const bool wt = P.lower_bc == 3;
    int jwt = NLEVSOI;
    if (wt) {
#pragma unroll 1
        for (int j = 1; j <= NLEVSOI; ++j)
            if (zwt <= k.zi(j)) { jwt = j - 1; break; }
    }

    double liq[N1], smp[N1], hk[N1], qout[N1], dqodw1[N1], dqodw2[N1], fn1[N1];
    double d[N1], du[N1], dl2[N1], b[N1];
#pragma unroll 1
    for (int j = 1; j <= nl; ++j) liq[j] = k.ss(io.h2osoi_liq, j);

    int nsub = 0;
    bool done = false;
    double dtsub = P.dtime, dtdone = 0.0, qcharge = 0.0;
    double vwc_q = 0.0, imped_q = 1.0;          // compute_qcharge's level jwt+1 of the last trial
#pragma unroll 1
    for (int guard = 0; guard < P.max_trials; ++guard) {
        nsub = nsub + 1;
        // ---- level 1 suction, then stream the levels
        double s2c = rel_sat(k, 1, liq[1]);
        double smp_c, dsmpdw_c;
        suction(k, 1, s2c, smp_c, dsmpdw_c);
        double qin = qinfl, dqidw0 = 0.0, dqidw1 = 0.0;
        double hk_nl = 0.0, dhkdw_nl = 0.0;
        // pending dgtsv row: d_p, du_p, b_p; its sub-diagonal arrives with the next row
        double d_p = 0.0, du_p = 0.0, b_p = 0.0;
#pragma unroll 1
        for (int j = 1; j <= nl; ++j) {
            double s2n = 0.0, smp_n = 0.0, dsmpdw_n = 0.0;
            if (j < nl) {
                s2n = rel_sat(k, j + 1, liq[j + 1]);
                suction(k, j + 1, s2n, smp_n, dsmpdw_n);
            }
            double s1, imped;
            if (j == nl) {
                s1 = s2c;
                imped = pow10_dd(-P.e_ice * k.g(io.icefrac, j));
            } else {
                s1 = 0.5 * (s2c + s2n);
                imped = pow10_dd(-P.e_ice * (0.5 * (k.g(io.icefrac, j) + k.g(io.icefrac, j + 1))));
            }
            s1 = fmn(s1, 1.0);
            s1 = fmx(0.01, s1);
            const double ws = k.g(io.watsat, j), bsw = k.g(io.bsw, j);
            const double hkj = imped * k.g(io.hksat, j) * pow(s1, 2.0 * bsw + 3.0);
            const double dhkdw = (2.0 * bsw + 3.0) * hkj / s1;
            smp[j] = smp_c;
            hk[j] = hkj;
            if (wt && j == jwt + 1) {
                vwc_q = fmx(liq[j], 1.0e-6) / (k.ss(io.dz, j) * DENH2O);
                imped_q = imped;
            }
            // flux out of the bottom of level j and its derivatives
            double qo, dq1, dq2;
            if (j < nl) {
                const double dhkds1 = 0.5 * dhkdw / ws;
                const double dhkds2 = 0.5 * dhkdw / k.g(io.watsat, j + 1);
                const double num = smp_n - smp_c;
                const double den = M_TO_MM * (k.ss(io.z, j + 1) - k.ss(io.z, j));
                qo = -hkj * num / den + hkj;
                dq1 = (hkj * dsmpdw_c - dhkds1 * num) / den + dhkds1;
                dq2 = (-hkj * dsmpdw_n - dhkds2 * num) / den + dhkds2;
            } else if (P.lower_bc == 3) {            // bc_waterTable (nl == nlevsoi)
                if (NLEVSOI > jwt) {
                    qo = 0.0; dq1 = 0.0; dq2 = 0.0;
                } else {
                    const double dhkds1 = dhkdw / ws;
                    const double num = -smp_c;
                    const double den = M_TO_MM * (zwt - k.ss(io.z, j));
                    qo = -hkj * num / den + hkj;
                    dq1 = (hkj * dsmpdw_c - dhkds1 * num) / den + dhkds1;
                    dq2 = 0.0;
                }
            } else if (P.lower_bc == 1) {            // bc_flux: free drainage
                qo = hkj; dq1 = dhkdw / ws; dq2 = 0.0;
            } else {                                 // bc_zero_flux
                qo = 0.0; dq1 = 0.0; dq2 = 0.0;
            }
            qout[j] = qo; dqodw1[j] = dq1; dqodw2[j] = dq2;
            if (j == nl) { hk_nl = hkj; dhkdw_nl = dhkdw; }
            // tridiagonal row j
            const double dt_dz = dtsub / (M_TO_MM * k.ss(io.dz, j));
            const double amx = (j == 1) ? 0.0 : dqidw0 * dt_dz;
            const double bmx = -1.0 - (-dqidw1 + dq1) * dt_dz;
            const double cmx = (j == nl) ? 0.0 : -dq2 * dt_dz;
            const double fluxNet = qin - qo - k.g(io.qflx_rootsoi, j);
            fn1[j] = fluxNet;
            const double rmx = -fluxNet * dt_dz;
            if (j == 1) {
                d_p = bmx; du_p = cmx; b_p = rmx;
            } else {
                // dgtsv elimination step i = j-2 (0-based) on rows j-1 (pending) and j
                double dl = amx, dn = bmx, dun = cmx, bn = rmx;
                if (fabs(d_p) >= fabs(dl)) {
                    if (d_p == 0.0) return j - 1;
                    const double fact = dl / d_p;
                    dn = dn - fact * du_p;
                    bn = bn - fact * b_p;
                    dl2[j - 1] = 0.0;
                } else {
                    const double fact = d_p / dl;
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
            s2c = s2n; smp_c = smp_n; dsmpdw_c = dsmpdw_n;
        }
        if (d_p == 0.0) return nl;
        d[nl] = d_p; du[nl] = du_p; b[nl] = b_p;
        // back substitution (1-based rows here)
        b[nl] = b[nl] / d[nl];
        if (nl > 1) b[nl - 1] = (b[nl - 1] - du[nl - 1] * b[nl]) / d[nl - 1];
#pragma unroll 1
        for (int i = nl - 2; i >= 1; --i) b[i] = (b[i] - du[i] * b[i + 1] - dl2[i] * b[i + 2]) / d[i];
        // ---- error estimate (:1306-1348)
        double errorMax = 0.0;
#pragma unroll 1
        for (int j = 1; j <= nl; ++j) {
            const double dt_dz = dtsub / (M_TO_MM * k.ss(io.dz, j));
            double fluxNet0;
            if (P.expensive) {
                const double qi = (j == 1) ? qinfl : qout[j - 1];
                const double qin_test = (j == 1) ? qi + 0.0 * b[j]
                                                 : qi + dqodw1[j - 1] * b[j - 1] + dqodw2[j - 1] * b[j];
                const double qout_test = (j == nl) ? qout[j] + dqodw1[j] * b[j]
                                                   : qout[j] + dqodw1[j] * b[j] + dqodw2[j] * b[j + 1];
                fluxNet0 = qin_test - qout_test - k.g(io.qflx_rootsoi, j);
            } else {
                fluxNet0 = b[j] / dt_dz;
            }
            const double e = fabs(fn1[j] - fluxNet0) * dtsub * 0.5;
            errorMax = (j == 1) ? e : ((errorMax < e) ? e : errorMax);
        }
        if (errorMax > P.xTolerUpper && dtsub > P.dtmin) {
            dtsub = fmx(dtsub / 2.0, P.dtmin);
            continue;
        }
#pragma unroll 1
        for (int j = 1; j <= nl; ++j) liq[j] = liq[j] + b[j] * (M_TO_MM * k.ss(io.dz, j));
        double qcTemp;
        if (P.lower_bc == 1) qcTemp = hk_nl + dhkdw_nl * b[nl];
        else if (P.lower_bc == 2) qcTemp = 0.0;
        else qcTemp = qout[nl] + dqodw1[nl] * b[nl];
        qcharge = qcharge + qcTemp * (dtsub / P.dtime);
        dtdone = dtdone + dtsub;
        if (fabs(P.dtime - dtdone) < P.verySmall) { done = true; break; }
        if (errorMax < P.xTolerLower) dtsub = dtsub * 2.0;
        dtsub = fmn(dtsub, P.dtime - dtdone);
    }
    if (!done) return -1;
    io.num_substeps[c] = (double)nsub;
    // over-saturated layers pass their excess upward (:1405-1409)
#pragma unroll 1
    for (int j = nl; j >= 2; --j) {
        const double cap = k.g(io.eff_porosity, j) * M_TO_MM * k.ss(io.dz, j);
        const double over = fmx(liq[j] - cap, 0.0);
        liq[j] = fmn(cap, liq[j]);
        liq[j - 1] = liq[j - 1] + over;
    }
    double* h2osoi_liq = io.h2osoi_liq;
#pragma unroll 1
    for (int j = 1; j <= nl; ++j) {
        h2osoi_liq[c + (size_t)(j - LS) * k.ld] = liq[j];
        io.smp_l[c + (size_t)(j - 1) * k.ld] = smp[j];
        io.hk_l[c + (size_t)(j - 1) * k.ld] = hk[j];
        io.qin[c + (size_t)(j - 1) * k.ld] = (j == 1) ? qinfl : qout[j - 1];
        io.qout[c + (size_t)(j - 1) * k.ld] = qout[j];
    }
    // compute_qcharge for the water-table boundary (:2016-2135)
    if (wt && jwt < NLEVSOI) {
        const double wh_zwt = -k.g(io.sucsat, jwt + 1) - zwt * M_TO_MM;
        double s1 = fmx(vwc_q / k.g(io.watsat, jwt + 1), 0.01);
        s1 = fmn(1.0, s1);
        const double ka = imped_q * k.g(io.hksat, jwt + 1) * pow(s1, 2.0 * k.g(io.bsw, jwt + 1) + 3.0);
        const int jm = jwt > 1 ? jwt : 1;
        const double smp1 = fmx(io.smpmin[c], smp[jm]);
        const double wh = smp1 - k.ss(io.z, jm) * M_TO_MM;
        if (jwt == 0) qcharge = -ka * (wh_zwt - wh) / ((zwt + (double)1.e-3f) * M_TO_MM);
        else qcharge = -ka * (wh_zwt - wh) / ((zwt - k.ss(io.z, jwt)) * M_TO_MM * 2.0);
        qcharge = fmx(-10.0 / P.dtime, qcharge);
        qcharge = fmn(10.0 / P.dtime, qcharge);
    }
    io.qcharge[c] = qcharge;
    return 0;
}

__global__ void __launch_bounds__(128)
moisture_form_kernel(ctsmg_soilwater_io io, int begc, int nfilt, const int32_t* __restrict__ filt,
                     MoistureFormArgs P, DevError* err) {
    const int fc = blockIdx.x * blockDim.x + threadIdx.x;
    if (fc >= nfilt) return;
    const int cg = filt ? filt[fc] : fc + begc;
    const int info = mf_column(io, cg - begc, P);
    if (info > 0) report_error(err, cg, info, CTSMG_E_SINGULAR);
    else if (info < 0) report_error(err, cg, 0, CTSMG_E_TIMEOUT);
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
template <bool HYDRO>
__global__ void __launch_bounds__(128)
mf_step_kernel(ctsmg_soilwater_io io, int ncol, MoistureFormArgs P, int flexcn, int refresh, DevError* err,
               const int32_t* __restrict__ filt, HydroStepArgs hy) {
    const int fc = blockIdx.x * blockDim.x + threadIdx.x;
    if (fc >= ncol) return;
    const int c = filt ? filt[fc] - 1 : fc;
    ctsmg_soilhydrology_params hp = hy.par;
    if (HYDRO) {
        if (hy.baseflow_scalar_c) hp.baseflow_scalar = hy.baseflow_scalar_c[c];
        if (hy.fff_c) hp.fff = hy.fff_c[c];
    }
    set_soil_water_fractions(io, c);
    if (HYDRO) {
        hydro::saturated_excess_runoff(hy.io, c, hp.fff);
        hydro::infiltration_chain(hy.io, c, hp, P.dtime);    // qflx_infl for SoilWater
    }
    const int info = mf_column(io, c, P);
    if (info > 0) report_error(err, c + 1, info, CTSMG_E_SINGULAR);
    else if (info < 0) report_error(err, c + 1, 0, CTSMG_E_TIMEOUT);
    if (flexcn) flexcn_column(io, c);
    if (HYDRO) {
        hydro::perched_water_table(hy.io, c);
        hydro::theta_based_water_table(hy.io, c);
        hydro::perched_lateral_flow(hy.io, c, hp, P.dtime);
        hydro::subsurface_lateral_flow(hy.io, c, hp, P.dtime);
    }
    if (refresh) refresh_h2osoi_vol(io, c);
}

cudaError_t launch_mf_step(const ctsmg_soilwater_io& io, int ncol, const MoistureFormArgs& P, int flexcn, int refresh,
                           DevError* err, const int32_t* d_filt, cudaStream_t s, const HydroStepArgs* hy) {
    if (ncol <= 0) return cudaSuccess;
    if (hy)
        mf_step_kernel<true><<<(ncol + 127) / 128, 128, 0, s>>>(io, ncol, P, flexcn, refresh, err, d_filt, *hy);
    else
        mf_step_kernel<false><<<(ncol + 127) / 128, 128, 0, s>>>(io, ncol, P, flexcn, refresh, err, d_filt,
                                                                HydroStepArgs{});
    return cudaGetLastError();
}

cudaError_t launch_moisture_form(const ctsmg_soilwater_io& io, int begc, int nfilt, const int32_t* d_filt,
                                 const MoistureFormArgs& P, DevError* err, cudaStream_t s) {
    if (nfilt <= 0) return cudaSuccess;
    moisture_form_kernel<<<(nfilt + 127) / 128, 128, 0, s>>>(io, begc, nfilt, d_filt, P, err);
    return cudaGetLastError();
}

cudaError_t launch_flexcn(const ctsmg_soilwater_io& io, int begc, int nfilt, const int32_t* d_filt, cudaStream_t s) {
    if (nfilt <= 0) return cudaSuccess;
    flexcn_kernel<<<(nfilt + 127) / 128, 128, 0, s>>>(io, begc, nfilt, d_filt);
    return cudaGetLastError();
}

} // namespace ctsmg
