// ctsm_oracle_mf.cpp -- CPU oracle (test infrastructure only): the moisture
// form of SoilWater (soilwater_movement_method = 1) and the use_flexibleCN
// negative-liquid fix that SoilWater applies after either form.
//
// Follows src/biogeophys/SoilWaterMovementMod.F90 statement by statement:
//   soilwater_moisture_form              :976-1440
//   compute_hydraulic_properties         :1444-1556
//   compute_moisture_fluxes_and_derivs   :1560-1866
//   compute_RHS_moisture_form            :1871-1937
//   compute_LHS_moisture_form            :1941-2012
//   compute_qcharge                      :2016-2135
//   IceImpedance                         :2139-2160
//   SoilWater (flexibleCN fix)           :331-368
// with the Clapp-Hornberger curve (SoilWaterRetentionCurveClappHornberg1978Mod.F90:45-125).
// The tridiagonal solve is LAPACK dgtsv (Gaussian elimination with partial
// pivoting, NRHS = 1), restated from the published reference-LAPACK
// algorithm; the LAPACK the reference links is unpinned, so the CPU tests
// check this restatement against scipy.linalg.lapack.dgtsv.
// Parity is unpinned: the reference ships no test of these routines.
#include <cmath>
#include <cstdint>
#include <algorithm>
#include "ctsm_gpu.h"
#include "ctsm_oracle.h"
#include "oracle_libm.h"

namespace {

const double DENH2O = 1.000e3;
const double DENICE = 0.917e3;
const double M_TO_MM = 1.e3;
const int NLEVSNO = CTSMG_NLEVSNO;
const int NLEVSOI = CTSMG_NLEVSOI;
const int LS = -NLEVSNO + 1;

using oracle_libm::o_pow;

struct Col {
    const ctsmg_soilwater_io* io;
    int c;
    int ld;
    double ss(const double* b, int j) const { return b[c + (size_t)(j - LS) * ld]; }
    double g(const double* b, int j) const { return b[c + (size_t)(j - 1) * ld]; }
    double zi(int j) const { return io->zi[c + (size_t)(j + NLEVSNO) * ld]; }
    double& ssw(double* b, int j) const { return b[c + (size_t)(j - LS) * ld]; }
    double& gw(double* b, int j) const { return b[c + (size_t)(j - 1) * ld]; }
};

// soil_hk / soil_suction of the Clapp-Hornberger curve
inline void ch78_hk(double hksat, double bsw, double s, double imped, double* hk, double* dhkds) {
    *hk = imped * hksat * o_pow(s, 2.0 * bsw + 3.0);
    if (dhkds) *dhkds = (2.0 * bsw + 3.0) * *hk / s;
}
inline void ch78_suction(double sucsat, double bsw, double s, double* smp, double* dsmpds) {
    *smp = -sucsat * o_pow(s, -bsw);
    if (dsmpds) *dsmpds = -bsw * *smp / s;
}

} // namespace

// dgtsv, NRHS = 1: dl(1:n-1), d(1:n), du(1:n-1), b(1:n) as 0-based arrays.
// Returns info (0, or the 1-based index of the zero pivot).
extern "C" int oracle_dgtsv(int n, double* dl, double* d, double* du, double* b) {
    if (n <= 0) return n < 0 ? -1 : 0;
    for (int i = 0; i < n - 2; ++i) {
        if (std::fabs(d[i]) >= std::fabs(dl[i])) {
            if (d[i] == 0.0) return i + 1;
            const double fact = dl[i] / d[i];
            d[i + 1] = d[i + 1] - fact * du[i];
            b[i + 1] = b[i + 1] - fact * b[i];
            dl[i] = 0.0;
        } else {
            const double fact = d[i] / dl[i];
            d[i] = dl[i];
            double temp = d[i + 1];
            d[i + 1] = du[i] - fact * temp;
            dl[i] = du[i + 1];
            du[i + 1] = -fact * dl[i];
            du[i] = temp;
            temp = b[i];
            b[i] = b[i + 1];
            b[i + 1] = temp - fact * b[i + 1];
        }
    }
    if (n > 1) {
        const int i = n - 2;
        if (std::fabs(d[i]) >= std::fabs(dl[i])) {
            if (d[i] == 0.0) return i + 1;
            const double fact = dl[i] / d[i];
            d[i + 1] = d[i + 1] - fact * du[i];
            b[i + 1] = b[i + 1] - fact * b[i];
        } else {
            const double fact = d[i] / dl[i];
            d[i] = dl[i];
            double temp = d[i + 1];
            d[i + 1] = du[i] - fact * temp;
            du[i] = temp;
            temp = b[i];
            b[i] = b[i + 1];
            b[i + 1] = temp - fact * b[i + 1];
        }
    }
    if (d[n - 1] == 0.0) return n;
    b[n - 1] = b[n - 1] / d[n - 1];
    if (n > 1) b[n - 2] = (b[n - 2] - du[n - 2] * b[n - 1]) / d[n - 2];
    for (int i = n - 3; i >= 0; --i) b[i] = (b[i] - du[i] * b[i + 1] - dl[i] * b[i + 2]) / d[i];
    return 0;
}

namespace {

// One column of soilwater_moisture_form; returns 0 or the dgtsv info.
int mf_column(const Col& k, double e_ice, double dtime, const ctsmg_soilwater_movement_nml& nml) {
    const ctsmg_soilwater_io* io = k.io;
    const int c = k.c;
    const int nlayers = io->nbedrock[c];
    const int N1 = NLEVSOI + 2;
    double vwc_liq[N1], dt_dz[N1], hk[N1], smp[N1], dhkdw[N1], dsmpdw[N1], imped[N1];
    double qin[N1], qout[N1], dqidw0[N1], dqidw1[N1], dqodw1[N1], dqodw2[N1];
    double amx[N1], bmx[N1], cmx[N1], rmx[N1], dwat[N1];
    double fluxNet0[N1], fluxNet1[N1];
    const bool expensive = nml.flux_calculation == 42;
    const int lbc = nml.lower_boundary_condition;
    const double zwt = io->zwt[c];

    int nsubstep = 0;
    double dtsub = dtime, dtdone = 0.0;
    double qcharge = 0.0;
    for (;;) {
        nsubstep = nsubstep + 1;
        for (int j = 1; j <= nlayers; ++j) {
            vwc_liq[j] = std::max(k.ss(io->h2osoi_liq, j), 1.0e-6) / (k.ss(io->dz, j) * DENH2O);
            dt_dz[j] = dtsub / (M_TO_MM * k.ss(io->dz, j));
        }
        // compute_hydraulic_properties
        double s2[N1];
        for (int j = 1; j <= nlayers; ++j) {
            s2[j] = vwc_liq[j] / k.g(io->watsat, j);
            s2[j] = std::min(s2[j], 1.0);
            s2[j] = std::max(0.01, s2[j]);
        }
        for (int j = 1; j <= nlayers; ++j) {
            double s1;
            if (j == nlayers) {
                s1 = s2[j];
                imped[j] = o_pow(10.0, -e_ice * k.g(io->icefrac, j));
            } else {
                s1 = 0.5 * (s2[j] + s2[j + 1]);
                imped[j] = o_pow(10.0, -e_ice * (0.5 * (k.g(io->icefrac, j) + k.g(io->icefrac, j + 1))));
            }
            s1 = std::min(s1, 1.0);
            s1 = std::max(0.01, s1);
            double dhkds, dsmpds;
            ch78_hk(k.g(io->hksat, j), k.g(io->bsw, j), s1, imped[j], &hk[j], &dhkds);
            ch78_suction(k.g(io->sucsat, j), k.g(io->bsw, j), s2[j], &smp[j], &dsmpds);
            dhkdw[j] = dhkds;
            dsmpdw[j] = dsmpds / k.g(io->watsat, j);
            k.gw(io->smp_l, j) = smp[j];
            k.gw(io->hk_l, j) = hk[j];
        }
        // compute_moisture_fluxes_and_derivs (upper boundary bc_flux)
        for (int j = 1; j <= nlayers; ++j) qin[j] = qout[j] = dqidw0[j] = dqidw1[j] = dqodw1[j] = dqodw2[j] = 0.0;
        {
            const int j = 1;
            qin[j] = io->qflx_infl[c];
            dqidw1[j] = 0.0;
            const double dhkds1 = 0.5 * dhkdw[j] / k.g(io->watsat, j);
            const double dhkds2 = 0.5 * dhkdw[j] / k.g(io->watsat, j + 1);
            const double num = smp[j + 1] - smp[j];
            const double den = M_TO_MM * (k.ss(io->z, j + 1) - k.ss(io->z, j));
            qout[j] = -hk[j] * num / den + hk[j];
            dqodw1[j] = (hk[j] * dsmpdw[j] - dhkds1 * num) / den + dhkds1;
            dqodw2[j] = (-hk[j] * dsmpdw[j + 1] - dhkds2 * num) / den + dhkds2;
        }
        for (int j = 2; j <= nlayers - 1; ++j) {
            qin[j] = qout[j - 1];
            dqidw0[j] = dqodw1[j - 1];
            dqidw1[j] = dqodw2[j - 1];
            const double dhkds1 = 0.5 * dhkdw[j] / k.g(io->watsat, j);
            const double dhkds2 = 0.5 * dhkdw[j] / k.g(io->watsat, j + 1);
            const double num = smp[j + 1] - smp[j];
            const double den = M_TO_MM * (k.ss(io->z, j + 1) - k.ss(io->z, j));
            qout[j] = -hk[j] * num / den + hk[j];
            dqodw1[j] = (hk[j] * dsmpdw[j] - dhkds1 * num) / den + dhkds1;
            dqodw2[j] = (-hk[j] * dsmpdw[j + 1] - dhkds2 * num) / den + dhkds2;
        }
        {
            int j = nlayers;
            qin[j] = qout[j - 1];
            dqidw0[j] = dqodw1[j - 1];
            dqidw1[j] = dqodw2[j - 1];
            if (lbc == 3) {                       // bc_waterTable (nlayers == nlevsoi)
                int jwt = NLEVSOI;
                for (int jj = 1; jj <= NLEVSOI; ++jj)
                    if (zwt <= k.zi(jj)) { jwt = jj - 1; break; }
                j = NLEVSOI;
                if (j > jwt) {
                    qout[j] = 0.0; dqodw1[j] = 0.0; dqodw2[j] = 0.0;
                } else {
                    const double dhkds1 = dhkdw[j] / k.g(io->watsat, j);
                    const double num = -smp[j];
                    const double den = M_TO_MM * (zwt - k.ss(io->z, j));
                    qout[j] = -hk[j] * num / den + hk[j];
                    dqodw1[j] = (hk[j] * dsmpdw[j] - dhkds1 * num) / den + dhkds1;
                    dqodw2[j] = 0.0;
                }
            } else if (lbc == 1) {                // bc_flux: free drainage
                qout[j] = hk[j];
                dqodw1[j] = dhkdw[j] / k.g(io->watsat, j);
            } else {                              // bc_zero_flux
                qout[j] = 0.0;
                dqodw1[j] = 0.0;
            }
        }
        // compute_RHS_moisture_form (non-iterative)
        for (int j = 1; j <= nlayers; ++j) {
            const double fluxNet = qin[j] - qout[j] - k.g(io->qflx_rootsoi, j);
            rmx[j] = -fluxNet * dt_dz[j];
        }
        // compute_LHS_moisture_form
        amx[1] = 0.0;
        bmx[1] = -1.0 - (-dqidw1[1] + dqodw1[1]) * dt_dz[1];
        cmx[1] = -dqodw2[1] * dt_dz[1];
        for (int j = 2; j <= nlayers - 1; ++j) {
            amx[j] = dqidw0[j] * dt_dz[j];
            bmx[j] = -1.0 - (-dqidw1[j] + dqodw1[j]) * dt_dz[j];
            cmx[j] = -dqodw2[j] * dt_dz[j];
        }
        amx[nlayers] = dqidw0[nlayers] * dt_dz[nlayers];
        bmx[nlayers] = -1.0 - (-dqidw1[nlayers] + dqodw1[nlayers]) * dt_dz[nlayers];
        cmx[nlayers] = 0.0;
        // dgtsv on copies (:1277-1300)
        double dLow[N1], diag[N1], dUpp[N1];
        for (int i = 0; i < nlayers - 1; ++i) { dLow[i] = amx[i + 2]; dUpp[i] = cmx[i + 1]; }
        for (int i = 0; i < nlayers; ++i) { diag[i] = bmx[i + 1]; dwat[i + 1] = rmx[i + 1]; }
        const int info = oracle_dgtsv(nlayers, dLow, diag, dUpp, dwat + 1);
        if (info != 0) return info;
        // error estimate (:1306-1348)
        for (int j = 1; j <= nlayers; ++j) {
            if (expensive) {
                double qin_test, qout_test;
                if (j == 1) qin_test = qin[j] + dqidw1[j] * dwat[j];
                else qin_test = qin[j] + dqidw0[j] * dwat[j - 1] + dqidw1[j] * dwat[j];
                if (j == nlayers) qout_test = qout[j] + dqodw1[j] * dwat[j];
                else qout_test = qout[j] + dqodw1[j] * dwat[j] + dqodw2[j] * dwat[j + 1];
                fluxNet0[j] = qin_test - qout_test - k.g(io->qflx_rootsoi, j);
            } else {
                fluxNet0[j] = dwat[j] / dt_dz[j];
            }
            fluxNet1[j] = qin[j] - qout[j] - k.g(io->qflx_rootsoi, j);
        }
        double errorMax = std::fabs(fluxNet1[1] - fluxNet0[1]) * dtsub * 0.5;
        for (int j = 2; j <= nlayers; ++j)
            errorMax = std::max(errorMax, std::fabs(fluxNet1[j] - fluxNet0[j]) * dtsub * 0.5);
        if (errorMax > nml.xTolerUpper && dtsub > nml.dtmin) {
            dtsub = std::max(dtsub / 2.0, nml.dtmin);
            continue;
        }
        for (int j = 1; j <= nlayers; ++j)
            k.ssw(io->h2osoi_liq, j) = k.ss(io->h2osoi_liq, j) + dwat[j] * (M_TO_MM * k.ss(io->dz, j));
        double qcTemp;
        if (lbc == 1) qcTemp = hk[nlayers] + dhkdw[nlayers] * dwat[nlayers];
        else if (lbc == 2) qcTemp = 0.0;
        else qcTemp = qout[nlayers] + dqodw1[nlayers] * dwat[nlayers];
        qcharge = qcharge + qcTemp * (dtsub / dtime);
        dtdone = dtdone + dtsub;
        if (std::fabs(dtime - dtdone) < nml.verySmall) break;
        if (errorMax < nml.xTolerLower) dtsub = dtsub * 2.0;
        dtsub = std::min(dtsub, dtime - dtdone);
    }
    io->num_substeps[c] = (double)nsubstep;
    // over-saturated layers pass their excess upward (:1405-1409)
    for (int j = nlayers; j >= 2; --j) {
        const double cap = k.g(io->eff_porosity, j) * M_TO_MM * k.ss(io->dz, j);
        const double over = std::max(k.ss(io->h2osoi_liq, j) - cap, 0.0);
        k.ssw(io->h2osoi_liq, j) = std::min(cap, k.ss(io->h2osoi_liq, j));
        k.ssw(io->h2osoi_liq, j - 1) = k.ss(io->h2osoi_liq, j - 1) + over;
    }
    for (int j = 1; j <= nlayers; ++j) {
        k.gw(io->qin, j) = qin[j];
        k.gw(io->qout, j) = qout[j];
    }
    // compute_qcharge for the water-table boundary (:1425-1436, 2016-2135)
    if (lbc == 3) {
        int jwt = NLEVSOI;
        for (int j = 1; j <= NLEVSOI; ++j)
            if (zwt <= k.zi(j)) { jwt = j - 1; break; }
        if (jwt < NLEVSOI) {
            const double wh_zwt = -k.g(io->sucsat, jwt + 1) - zwt * M_TO_MM;
            double s1 = std::max(vwc_liq[jwt + 1] / k.g(io->watsat, jwt + 1), 0.01);
            s1 = std::min(1.0, s1);
            double ka;
            ch78_hk(k.g(io->hksat, jwt + 1), k.g(io->bsw, jwt + 1), s1, imped[jwt + 1], &ka, nullptr);
            const double smp1 = std::max(io->smpmin[c], smp[std::max(1, jwt)]);
            const double wh = smp1 - k.ss(io->z, std::max(1, jwt)) * M_TO_MM;
            if (jwt == 0) qcharge = -ka * (wh_zwt - wh) / ((zwt + (double)1.e-3f) * M_TO_MM);
            else qcharge = -ka * (wh_zwt - wh) / ((zwt - k.ss(io->z, jwt)) * M_TO_MM * (double)2.0f);
            qcharge = std::max(-10.0 / dtime, qcharge);
            qcharge = std::min(10.0 / dtime, qcharge);
        }
    }
    io->qcharge[c] = qcharge;
    return 0;
}

} // namespace

// soilwater_moisture_form over the filter.  Returns 0, or CTSMG_E_SINGULAR
// with *err_col = the 1-based column whose dgtsv failed.
extern "C" int oracle_soilwater_mf(const ctsmg_bounds* bounds, int num_hydrologyc, const int32_t* filter_hydrologyc,
                                   const ctsmg_soilwater_io* io, double e_ice, double dtime,
                                   const ctsmg_soilwater_movement_nml* nml, int* err_col) {
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(max : bad)
    for (int fc = 0; fc < num_hydrologyc; ++fc) {
        Col k{io, filter_hydrologyc[fc] - bounds->begc, io->ldc};
        if (mf_column(k, e_ice, dtime, *nml) != 0) bad = std::max(bad, filter_hydrologyc[fc]);
    }
    if (err_col) *err_col = bad;
    return bad ? CTSMG_E_SINGULAR : 0;
}

// The use_flexibleCN fix SoilWater applies after either form (:331-368):
// negative liquid borrowed from the layer below, the bottom layer topped up
// from the aquifer, and h2osoi_vol refreshed.
extern "C" void oracle_flexcn_fix(const ctsmg_bounds* bounds, int num_hydrologyc, const int32_t* filter_hydrologyc,
                                  const ctsmg_soilwater_io* io) {
    const double watmin = 0.001;
    for (int fc = 0; fc < num_hydrologyc; ++fc) {
        Col k{io, filter_hydrologyc[fc] - bounds->begc, io->ldc};
        for (int j = 1; j <= NLEVSOI - 1; ++j) {
            const double liq = k.ss(io->h2osoi_liq, j);
            const double xs = liq < 0.0 ? watmin - liq : 0.0;
            k.ssw(io->h2osoi_liq, j) = liq + xs;
            k.ssw(io->h2osoi_liq, j + 1) = k.ss(io->h2osoi_liq, j + 1) - xs;
        }
        const double liq = k.ss(io->h2osoi_liq, NLEVSOI);
        const double xs = liq < watmin ? watmin - liq : 0.0;
        k.ssw(io->h2osoi_liq, NLEVSOI) = liq + xs;
        io->wa[k.c] = io->wa[k.c] - xs;
        for (int j = 1; j <= NLEVSOI; ++j)
            k.gw(const_cast<double*>(io->h2osoi_vol), j) =
                k.ss(io->h2osoi_liq, j) / (k.ss(io->dz, j) * DENH2O) + k.ss(io->h2osoi_ice, j) / (k.ss(io->dz, j) * DENICE);
    }
}

// SetSoilWaterFractions (src/biogeophys/SoilHydrologyMod.F90:236-249) with no
// excess ice: eff_porosity and icefrac on levels 1..nlevsoi.
extern "C" void oracle_set_soil_water_fractions(const ctsmg_bounds* bounds, int num_hydrologyc,
                                                const int32_t* filter_hydrologyc, const ctsmg_soilwater_io* io) {
    const double excess_ice = 0.0;
    for (int j = 1; j <= NLEVSOI; ++j)
        for (int fc = 0; fc < num_hydrologyc; ++fc) {
            Col k{io, filter_hydrologyc[fc] - bounds->begc, io->ldc};
            const double dz_ext = k.ss(io->dz, j) + excess_ice / DENICE;
            const double vol_ice = std::min(k.g(io->watsat, j), (k.ss(io->h2osoi_ice, j) + excess_ice) / (dz_ext * DENICE));
            k.gw(const_cast<double*>(io->eff_porosity), j) = std::max(0.01, k.g(io->watsat, j) - vol_ice);
            k.gw(io->icefrac, j) = std::min(1.0, vol_ice / k.g(io->watsat, j));
        }
}

