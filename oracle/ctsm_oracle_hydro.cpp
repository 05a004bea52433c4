// ctsm_oracle_hydro.cpp -- CPU oracle (test infrastructure only) of the
// water-table and drainage routines of the default hydrology, for natural
// soil columns outside hillslopes, statement by statement:
//   SaturatedExcessRunoff / ComputeFsatTopmodel  SaturatedExcessRunoffMod.F90:200-360
//   SetQflxInputs, RouteInfiltrationExcess, Infiltration  SoilHydrologyMod.F90:298-457
//   InfiltrationExcessRunoff (hksat qinmax)  InfiltrationExcessRunoffMod.F90:196-304
//   UpdateH2osfc, QflxH2osfcSurf, QflxH2osfcDrain  SurfaceWaterMod.F90:345-556
//   truncate_small_values   src/utils/NumericsMod.F90:50-99 (rel_epsilon 1e-13)
//   PerchedWaterTable       SoilHydrologyMod.F90:1525-1641
//   ThetaBasedWaterTable    SoilHydrologyMod.F90:1933-2025
//   PerchedLateralFlow      SoilHydrologyMod.F90:1645-1929
//   SubsurfaceLateralFlow   SoilHydrologyMod.F90:2029-2565
//   WaterTable, Drainage    SoilHydrologyMod.F90:607-1410 (aquifer layer, non-VIC)
// sat_lev = 0.9 is a default-real literal in the reference, reproduced as
// (double)0.9f.  Parity unpinned: the reference ships no test of these.
#include <cmath>
#include <cstdint>
#include <algorithm>
#include "ctsm_gpu.h"
#include "ctsm_oracle.h"
#include "oracle_libm.h"

namespace {
const double TFRZ = 273.15, DENH2O = 1.000e3, DENICE = 0.917e3;
const double WATMIN = 0.01, PONDMX = 0.0, RPI = 3.14159265358979323846, AQUIFER_WATER_BASELINE = 5000.0;
const int NLEVSNO = CTSMG_NLEVSNO, NLEVSOI = CTSMG_NLEVSOI, LS = -NLEVSNO + 1;
using oracle_libm::o_pow;
using oracle_libm::o_exp;

struct K {
    const ctsmg_hydrology_io* io;
    int c, ld;
    double& liq(int j) const { return io->h2osoi_liq[c + (size_t)(j - LS) * ld]; }
    double& ice(int j) const { return io->h2osoi_ice[c + (size_t)(j - LS) * ld]; }
    double dz(int j) const { return io->dz[c + (size_t)(j - LS) * ld]; }
    double z(int j) const { return io->z[c + (size_t)(j - LS) * ld]; }
    double t(int j) const { return io->t_soisno[c + (size_t)(j - LS) * ld]; }
    double zi(int j) const { return io->zi[c + (size_t)(j + NLEVSNO) * ld]; }
    double watsat(int j) const { return io->watsat[c + (size_t)(j - 1) * ld]; }
    double hksat(int j) const { return io->hksat[c + (size_t)(j - 1) * ld]; }
    double bsw(int j) const { return io->bsw[c + (size_t)(j - 1) * ld]; }
    double sucsat(int j) const { return io->sucsat[c + (size_t)(j - 1) * ld]; }
    double eff(int j) const { return io->eff_porosity[c + (size_t)(j - 1) * ld]; }
    double& vol(int j) const { return io->h2osoi_vol[c + (size_t)(j - 1) * ld]; }
    double& icefrac(int j) const { return io->icefrac[c + (size_t)(j - 1) * ld]; }
};
int jwt_of(const K& k, double zwt) {
    int jwt = NLEVSOI;
    for (int j = 1; j <= NLEVSOI; ++j)
        if (zwt <= k.zi(j)) { jwt = j - 1; break; }
    return jwt;
}

double syield(const K& k, int j, double depth, double aq_min) {
    double s_y = k.watsat(j) * (1. - o_pow(1. + 1.e3 * depth / k.sucsat(j), -1. / k.bsw(j)));
    return std::max(s_y, aq_min);
}

// WaterTable (SoilHydrologyMod.F90:607-861)
void water_table(const K& k, const ctsmg_hydrology_io* io, const ctsmg_soilhydrology_params* P, double dtime) {
    const int c = k.c;
    const double sat_lev_r8 = (double)0.9f;
    io->qflx_drain[c] = 0.0;
    io->qflx_rsub_sat[c] = 0.0;
    io->qflx_drain_perched[c] = 0.0;
    int jwt = jwt_of(k, io->zwt[c]);
    const double rous = syield(k, NLEVSOI, io->zwt[c], P->aq_sp_yield_min);
    if (jwt == NLEVSOI) {
        io->wa[c] = io->wa[c] + io->qcharge[c] * dtime;
        io->zwt[c] = io->zwt[c] - (io->qcharge[c] * dtime) / 1000.0 / rous;
    } else {
        double qcharge_tot = io->qcharge[c] * dtime;
        if (qcharge_tot > 0.) {
            for (int j = jwt + 1; j >= 1; --j) {
                const double s_y = syield(k, j, io->zwt[c], P->aq_sp_yield_min);
                double layer = std::min(qcharge_tot, (s_y * (io->zwt[c] - k.zi(j - 1)) * 1.e3));
                layer = std::max(layer, 0.0);
                if (s_y > 0.0) io->zwt[c] = io->zwt[c] - layer / s_y / 1000.0;
                qcharge_tot = qcharge_tot - layer;
                if (qcharge_tot <= 0.) break;
            }
        } else {
            for (int j = jwt + 1; j <= NLEVSOI; ++j) {
                const double s_y = syield(k, j, io->zwt[c], P->aq_sp_yield_min);
                double layer = std::max(qcharge_tot, -(s_y * (k.zi(j) - io->zwt[c]) * 1.e3));
                layer = std::min(layer, 0.0);
                qcharge_tot = qcharge_tot - layer;
                if (qcharge_tot >= 0.) {
                    io->zwt[c] = io->zwt[c] - layer / s_y / 1000.0;
                    break;
                } else {
                    io->zwt[c] = k.zi(j);
                }
            }
            if (qcharge_tot > 0.) io->zwt[c] = io->zwt[c] - qcharge_tot / 1000.0 / rous;
        }
        jwt = jwt_of(k, io->zwt[c]);
    }
    int k_frz = (k.t(1) > TFRZ) ? NLEVSOI : 1;
    for (int kk = 2; kk <= NLEVSOI; ++kk)
        if (k.t(kk - 1) > TFRZ && k.t(kk) <= TFRZ) { k_frz = kk; break; }
    io->frost_table[c] = k.z(k_frz);
    io->zwt_perched[c] = io->frost_table[c];
    if (io->zwt[c] < io->frost_table[c] && k.t(k_frz) <= TFRZ) {
    } else {
        int k_perch = 1;
        for (int kk = k_frz; kk >= 1; --kk) {
            k.vol(kk) = k.liq(kk) / (k.dz(kk) * DENH2O) + k.ice(kk) / (k.dz(kk) * DENICE);
            if (k.vol(kk) / k.watsat(kk) <= sat_lev_r8) { k_perch = kk; break; }
        }
        if (k.t(k_frz) > TFRZ) k_perch = k_frz;
        if (k_frz > k_perch) {
            const double s1 = (k.liq(k_perch) / (k.dz(k_perch) * DENH2O) + k.ice(k_perch) / (k.dz(k_perch) * DENICE)) /
                              k.watsat(k_perch);
            const double s2 = (k.liq(k_perch + 1) / (k.dz(k_perch + 1) * DENH2O) +
                               k.ice(k_perch + 1) / (k.dz(k_perch + 1) * DENICE)) / k.watsat(k_perch + 1);
            const double m = (k.z(k_perch + 1) - k.z(k_perch)) / (s2 - s1);
            const double bb = k.z(k_perch + 1) - m * s2;
            io->zwt_perched[c] = std::max(0.0, m * sat_lev_r8 + bb);
        }
    }
}

// Drainage (SoilHydrologyMod.F90:864-1410), non-VIC
void drainage(const K& k, const ctsmg_hydrology_io* io, const ctsmg_soilhydrology_params* P, double dtime) {
    const int c = k.c;
    double dzmm[NLEVSOI + 1];
    for (int j = 1; j <= NLEVSOI; ++j) {
        dzmm[j] = k.dz(j) * 1.e3;
        const double vol_ice = std::min(k.watsat(j), k.ice(j) / (k.dz(j) * DENICE));
        k.icefrac(j) = std::min(1.0, vol_ice / k.watsat(j));
    }
    io->qflx_drain[c] = 0.0;
    io->qflx_rsub_sat[c] = 0.0;
    double rsub_top = 0.0;
    int jwt = jwt_of(k, io->zwt[c]);
    const double q_perch_max = P->perched_baseflow_scalar * std::sin(io->topo_slope[c] * (RPI / 180.0));
    int k_frz = (k.t(1) > TFRZ) ? NLEVSOI : 1;
    for (int kk = 2; kk <= NLEVSOI; ++kk)
        if (k.t(kk - 1) > TFRZ && k.t(kk) <= TFRZ) { k_frz = kk; break; }
    io->frost_table[c] = k.z(k_frz);
    io->zwt_perched[c] = io->frost_table[c];
    io->qflx_drain_perched[c] = 0.0;
    auto imped_k = [&](int kk) {
        return o_pow(10.0, -P->e_ice * (0.5 * (k.icefrac(kk) + k.icefrac(std::min(NLEVSOI, kk + 1)))));
    };
    if (io->zwt[c] < io->frost_table[c] && k.t(k_frz) <= TFRZ) {
        double wtsub = 0.0, q_perch = 0.0;
        for (int kk = jwt + 1; kk <= k_frz; ++kk) {
            q_perch = q_perch + imped_k(kk) * k.hksat(kk) * dzmm[kk];
            wtsub = wtsub + dzmm[kk];
        }
        if (wtsub > 0.0) q_perch = q_perch / wtsub;
        io->qflx_drain_perched[c] = q_perch_max * q_perch * (io->frost_table[c] - io->zwt[c]);
        double tot = -io->qflx_drain_perched[c] * dtime;
        for (int kk = jwt + 1; kk <= k_frz; ++kk) {
            double layer = std::max(tot, -(k.liq(kk) - WATMIN));
            layer = std::min(layer, 0.0);
            tot = tot - layer;
            k.liq(kk) = k.liq(kk) + layer;
            if (tot >= 0.) {
                io->zwt[c] = io->zwt[c] - layer / k.eff(kk) / 1000.0;
                break;
            } else {
                io->zwt[c] = k.zi(kk);
            }
        }
        io->qflx_drain_perched[c] = io->qflx_drain_perched[c] + tot / dtime;
        jwt = jwt_of(k, io->zwt[c]);
    } else {
        const double sat_lev = (double)0.9f;
        int k_perch = 1;
        for (int kk = k_frz; kk >= 1; --kk) {
            const double h2osoi_vol = k.liq(kk) / (k.dz(kk) * DENH2O) + k.ice(kk) / (k.dz(kk) * DENICE);
            if (h2osoi_vol / k.watsat(kk) <= sat_lev) { k_perch = kk; break; }
        }
        if (k.t(k_frz) > TFRZ) k_perch = k_frz;
        if (k_frz > k_perch) {
            const double s1 = (k.liq(k_perch) / (k.dz(k_perch) * DENH2O) + k.ice(k_perch) / (k.dz(k_perch) * DENICE)) /
                              k.watsat(k_perch);
            const double s2 = (k.liq(k_perch + 1) / (k.dz(k_perch + 1) * DENH2O) +
                               k.ice(k_perch + 1) / (k.dz(k_perch + 1) * DENICE)) / k.watsat(k_perch + 1);
            const double m = (k.z(k_perch + 1) - k.z(k_perch)) / (s2 - s1);
            const double bb = k.z(k_perch + 1) - m * s2;
            io->zwt_perched[c] = std::max(0.0, m * sat_lev + bb);
            double wtsub = 0.0, q_perch = 0.0;
            for (int kk = k_perch; kk <= k_frz; ++kk) {
                q_perch = q_perch + imped_k(kk) * k.hksat(kk) * dzmm[kk];
                wtsub = wtsub + dzmm[kk];
            }
            if (wtsub > 0.0) q_perch = q_perch / wtsub;
            io->qflx_drain_perched[c] = q_perch_max * q_perch * (io->frost_table[c] - io->zwt_perched[c]);
            double tot = -io->qflx_drain_perched[c] * dtime;
            for (int kk = k_perch + 1; kk <= k_frz; ++kk) {
                double layer = std::max(tot, -(k.liq(kk) - WATMIN));
                layer = std::min(layer, 0.0);
                tot = tot - layer;
                k.liq(kk) = k.liq(kk) + layer;
                if (tot >= 0.) {
                    io->zwt_perched[c] = io->zwt_perched[c] - layer / k.eff(kk) / 1000.0;
                    break;
                } else {
                    io->zwt_perched[c] = k.zi(kk);
                }
            }
            io->qflx_drain_perched[c] = io->qflx_drain_perched[c] + tot / dtime;
        } else {
            io->qflx_drain_perched[c] = 0.0;
        }
        const double fff = 1.0 / io->hkdepth[c];
        double dzsum = 0.0, icefracsum = 0.0;
        for (int j = std::max(jwt, 1); j <= NLEVSOI; ++j) {
            dzsum = dzsum + dzmm[j];
            icefracsum = icefracsum + k.icefrac(j) * dzmm[j];
        }
        const double imped = o_pow(10.0, -P->e_ice * (icefracsum / dzsum));
        const double rsub_top_max = 10.0 * std::sin((RPI / (double)180.f) * io->topo_slope[c]);
        rsub_top = imped * rsub_top_max * o_exp(-fff * io->zwt[c]);
        const double rous = syield(k, NLEVSOI, io->zwt[c], P->aq_sp_yield_min);
        if (jwt == NLEVSOI) {
            io->wa[c] = io->wa[c] - rsub_top * dtime;
            io->zwt[c] = io->zwt[c] + (rsub_top * dtime) / 1000.0 / rous;
            k.liq(NLEVSOI) = k.liq(NLEVSOI) + std::max(0.0, (io->wa[c] - AQUIFER_WATER_BASELINE));
            io->wa[c] = std::min(io->wa[c], AQUIFER_WATER_BASELINE);
        } else {
            double tot = -rsub_top * dtime;
            for (int j = jwt + 1; j <= NLEVSOI; ++j) {
                const double s_y = syield(k, j, io->zwt[c], P->aq_sp_yield_min);
                double layer = std::max(tot, -(s_y * (k.zi(j) - io->zwt[c]) * 1.e3));
                layer = std::min(layer, 0.0);
                k.liq(j) = k.liq(j) + layer;
                tot = tot - layer;
                if (tot >= 0.) {
                    io->zwt[c] = io->zwt[c] - layer / s_y / 1000.0;
                    break;
                } else {
                    io->zwt[c] = k.zi(j);
                }
            }
            io->zwt[c] = io->zwt[c] - tot / 1000.0 / rous;
            io->wa[c] = io->wa[c] + tot;
            jwt = jwt_of(k, io->zwt[c]);
        }
        io->zwt[c] = std::max(0.0, io->zwt[c]);
        io->zwt[c] = std::min(80.0, io->zwt[c]);
    }
    for (int j = NLEVSOI; j >= 2; --j) {
        const double xsi = std::max(k.liq(j) - k.eff(j) * dzmm[j], 0.0);
        k.liq(j) = std::min(k.eff(j) * dzmm[j], k.liq(j));
        k.liq(j - 1) = k.liq(j - 1) + xsi;
    }
    double xs1 = std::max(std::max(k.liq(1) - WATMIN, 0.0) -
                          std::max(0.0, (PONDMX + k.watsat(1) * dzmm[1] - k.ice(1) - WATMIN)), 0.0);
    k.liq(1) = k.liq(1) - xs1;
    if (P->h2osfcflag == 1) {
        io->h2osfc[c] = io->h2osfc[c] + xs1;
        io->qflx_rsub_sat[c] = 0.0;
    } else {
        io->qflx_rsub_sat[c] = xs1 / dtime;
    }
    xs1 = std::max(std::max(k.ice(1), 0.0) - std::max(0.0, (PONDMX + k.watsat(1) * dzmm[1] - k.liq(1))), 0.0);
    k.ice(1) = std::min(std::max(0.0, PONDMX + k.watsat(1) * dzmm[1] - k.liq(1)), k.ice(1));
    io->qflx_ice_runoff_xs[c] = xs1 / dtime;
    for (int j = 1; j <= NLEVSOI - 1; ++j) {
        double xs;
        if (k.liq(j) < WATMIN) {
            xs = WATMIN - k.liq(j);
            if (j == jwt) io->zwt[c] = io->zwt[c] + xs / k.eff(j) / 1000.0;
        } else {
            xs = 0.0;
        }
        k.liq(j) = k.liq(j) + xs;
        k.liq(j + 1) = k.liq(j + 1) - xs;
    }
    {
        const int j = NLEVSOI;
        double xs;
        if (k.liq(j) < WATMIN) {
            xs = WATMIN - k.liq(j);
            for (int i = NLEVSOI - 1; i >= 1; --i) {
                const double avail = std::max(k.liq(i) - WATMIN - xs, 0.0);
                if (avail >= xs) {
                    k.liq(j) = k.liq(j) + xs;
                    k.liq(i) = k.liq(i) - xs;
                    xs = 0.0;
                    break;
                } else {
                    k.liq(j) = k.liq(j) + avail;
                    k.liq(i) = k.liq(i) - avail;
                    xs = xs - avail;
                }
            }
        } else {
            xs = 0.0;
        }
        k.liq(j) = k.liq(j) + xs;
        rsub_top = rsub_top - xs / dtime;
    }
    io->qflx_drain[c] = io->qflx_rsub_sat[c] + rsub_top;
    io->qflx_qrgwl[c] = io->qflx_snwcp_liq[c];
}

} // namespace

extern "C" int oracle_hydrology(const ctsmg_bounds* b, int n, const int32_t* filt, const ctsmg_hydrology_io* io,
                                int which, const ctsmg_soilhydrology_params* P, double dtime) {
    const double sat_lev = (double)0.9f;
    for (int fc = 0; fc < n; ++fc) {
        const K k{io, filt[fc] - b->begc, io->ldc};
        const int c = k.c;
        if (which == 0) {                      // SaturatedExcessRunoff (TOPMODEL fsat)
            double fsat;
            if (io->frost_table[c] > io->zwt_perched[c] && io->frost_table[c] <= io->zwt[c])
                fsat = io->wtfact[c] * o_exp(-0.5 * P->fff * io->zwt_perched[c]);
            else
                fsat = io->wtfact[c] * o_exp(-0.5 * P->fff * io->zwt[c]);
            io->fsat[c] = fsat;
            io->qflx_sat_excess_surf[c] = fsat * io->qflx_rain_plus_snomelt[c];
            io->fcov[c] = fsat;
        } else if (which == 5) {               // SetQflxInputs .. Infiltration
            const double fh = io->frac_h2osfc[c];
            // SetQflxInputs (SoilHydrologyMod.F90:298-366)
            io->qflx_top_soil[c] = io->qflx_rain_plus_snomelt[c] + io->qflx_snow_h2osfc[c] + io->qflx_floodc[c];
            double fsno, qflx_evap;
            if (io->snl[c] >= 0) { fsno = 0.0; qflx_evap = io->qflx_liqevap_from_top_layer_col[c]; }
            else { fsno = io->frac_sno_eff[c]; qflx_evap = io->qflx_ev_soil_col[c]; }
            io->qflx_in_soil[c] = (1.0 - fh) * (io->qflx_top_soil[c] - io->qflx_sat_excess_surf[c]);
            io->qflx_top_soil_to_h2osfc[c] = fh * (io->qflx_top_soil[c] - io->qflx_sat_excess_surf[c]);
            io->qflx_in_soil[c] = io->qflx_in_soil[c] - (1.0 - fsno - fh) * qflx_evap;
            io->qflx_top_soil_to_h2osfc[c] = io->qflx_top_soil_to_h2osfc[c] - fh * io->qflx_ev_h2osfc_col[c];
            // InfiltrationExcessRunoff, hksat qinmax (InfiltrationExcessRunoffMod.F90:196-304)
            double qmu = 0.0;
            for (int j = 1; j <= 3; ++j) {
                const double q = o_pow(10.0, -P->e_ice * (io->icefrac[c + (size_t)(j - 1) * k.ld])) *
                                 io->hksat[c + (size_t)(j - 1) * k.ld];
                qmu = (j == 1) ? q : std::min(qmu, q);
            }
            io->qinmax[c] = (1.0 - io->fsat[c]) * qmu;
            io->qflx_infl_excess[c] = std::max(0.0, (io->qflx_in_soil[c] - (1.0 - fh) * io->qinmax[c]));
            // RouteInfiltrationExcess (:369-423)
            io->qflx_in_soil_limited[c] = io->qflx_in_soil[c] - io->qflx_infl_excess[c];
            if (P->h2osfcflag != 0) {
                io->qflx_in_h2osfc[c] = io->qflx_top_soil_to_h2osfc[c] + io->qflx_infl_excess[c];
                io->qflx_infl_excess_surf[c] = 0.0;
            } else {
                io->qflx_in_h2osfc[c] = io->qflx_top_soil_to_h2osfc[c];
                io->qflx_infl_excess_surf[c] = io->qflx_infl_excess[c];
            }
            // UpdateH2osfc (SurfaceWaterMod.F90:345-556)
            double frac_infclust = 0.0;
            if (P->h2osfcflag == 1) {
                if (io->frac_h2osfc_nosnow[c] <= P->pc) frac_infclust = 0.0;
                else frac_infclust = o_pow(io->frac_h2osfc_nosnow[c] - P->pc, P->mu);
            }
            if (io->h2osfc[c] > io->h2osfc_thresh[c] && P->h2osfcflag != 0) {
                const double k_wet = 1.0e-4 * std::sin((RPI / 180.0) * io->topo_slope[c]);
                io->qflx_h2osfc_surf[c] = k_wet * frac_infclust * (io->h2osfc[c] - io->h2osfc_thresh[c]);
                io->qflx_h2osfc_surf[c] = std::min(io->qflx_h2osfc_surf[c], (io->h2osfc[c] - io->h2osfc_thresh[c]) / dtime);
            } else {
                io->qflx_h2osfc_surf[c] = 0.0;
            }
            if (io->qflx_h2osfc_surf[c] < (double)1.0e-8f) io->qflx_h2osfc_surf[c] = 0.0;
            double h2osfc_partial = io->h2osfc[c] + (io->qflx_in_h2osfc[c] - io->qflx_h2osfc_surf[c]) * dtime;
            if (std::fabs(h2osfc_partial) < 1.e-13 * std::fabs(io->h2osfc[c])) h2osfc_partial = 0.0;
            if (h2osfc_partial < 0.0) {
                io->qflx_h2osfc_drain[c] = h2osfc_partial / dtime;
            } else {
                io->qflx_h2osfc_drain[c] = std::min(fh * io->qinmax[c], h2osfc_partial / dtime);
                if (P->h2osfcflag == 0) io->qflx_h2osfc_drain[c] = std::max(0.0, h2osfc_partial / dtime);
            }
            io->h2osfc[c] = h2osfc_partial - io->qflx_h2osfc_drain[c] * dtime;
            if (std::fabs(io->h2osfc[c]) < 1.e-13 * std::fabs(h2osfc_partial)) io->h2osfc[c] = 0.0;
            // Infiltration (:426-457)
            io->qflx_infl[c] = io->qflx_in_soil_limited[c] + io->qflx_h2osfc_drain[c];
        } else if (which == 6) {
            water_table(k, io, P, dtime);
        } else if (which == 7) {
            drainage(k, io, P, dtime);
        } else if (which == 1) {               // PerchedWaterTable
            int k_frz = (k.t(1) > TFRZ) ? NLEVSOI : 1;
            for (int kk = 2; kk <= NLEVSOI; ++kk)
                if (k.t(kk - 1) > TFRZ && k.t(kk) <= TFRZ) { k_frz = kk; break; }
            io->frost_table[c] = k.zi(k_frz - 1);
            io->zwt_perched[c] = io->frost_table[c];
            if (io->zwt[c] < io->frost_table[c] && k.t(k_frz) <= TFRZ) {
            } else if (k_frz > 1) {
                int k_perch = 1;
                for (int kk = k_frz; kk >= 1; --kk) {
                    k.vol(kk) = k.liq(kk) / (k.dz(kk) * DENH2O) + k.ice(kk) / (k.dz(kk) * DENICE);
                    if (k.vol(kk) / k.watsat(kk) <= sat_lev) { k_perch = kk; break; }
                }
                if (k.t(k_frz) > TFRZ) k_perch = k_frz;
                if (k_frz > k_perch) {
                    const double s1 = (k.liq(k_perch) / (k.dz(k_perch) * DENH2O) + k.ice(k_perch) / (k.dz(k_perch) * DENICE)) /
                                      k.watsat(k_perch);
                    const double s2 = (k.liq(k_perch + 1) / (k.dz(k_perch + 1) * DENH2O) +
                                       k.ice(k_perch + 1) / (k.dz(k_perch + 1) * DENICE)) / k.watsat(k_perch + 1);
                    if (s1 > s2) {
                        io->zwt_perched[c] = k.zi(k_perch - 1);
                    } else {
                        const double m = (k.z(k_perch + 1) - k.z(k_perch)) / (s2 - s1);
                        const double bb = k.z(k_perch + 1) - m * s2;
                        io->zwt_perched[c] = std::max(0.0, m * sat_lev + bb);
                    }
                }
            }
        } else if (which == 2) {               // ThetaBasedWaterTable
            const int nb = io->nbedrock[c];
            io->zwt[c] = k.zi(NLEVSOI);
            int k_zwt = nb, sat_flag = 1;
            for (int kk = nb; kk >= 1; --kk) {
                k.vol(kk) = k.liq(kk) / (k.dz(kk) * DENH2O) + k.ice(kk) / (k.dz(kk) * DENICE);
                if (k.vol(kk) / k.watsat(kk) <= sat_lev) { k_zwt = kk; sat_flag = 0; break; }
            }
            if (sat_flag == 1) k_zwt = 1;
            if (k_zwt == 1) {
                io->zwt[c] = k.zi(1);
            } else if (k_zwt < nb) {
                const double s1 = (k.liq(k_zwt) / (k.dz(k_zwt) * DENH2O) + k.ice(k_zwt) / (k.dz(k_zwt) * DENICE)) /
                                  k.watsat(k_zwt);
                const double s2 = (k.liq(k_zwt + 1) / (k.dz(k_zwt + 1) * DENH2O) +
                                   k.ice(k_zwt + 1) / (k.dz(k_zwt + 1) * DENICE)) / k.watsat(k_zwt + 1);
                const double m = (k.z(k_zwt + 1) - k.z(k_zwt)) / (s2 - s1);
                const double bb = k.z(k_zwt + 1) - m * s2;
                io->zwt[c] = std::max(0.0, m * sat_lev + bb);
            } else {
                io->zwt[c] = k.zi(nb);
            }
        } else if (which == 3) {               // PerchedLateralFlow
            const int nb = io->nbedrock[c];
            int k_frost = nb, k_perch = nb;
            for (int kk = 1; kk <= nb; ++kk)
                if (io->frost_table[c] >= k.zi(kk - 1) && io->frost_table[c] < k.zi(kk)) { k_frost = kk; break; }
            for (int kk = 1; kk <= nb; ++kk)
                if (io->zwt_perched[c] >= k.zi(kk - 1) && io->zwt_perched[c] < k.zi(kk)) { k_perch = kk; break; }
            io->qflx_drain_perched[c] = 0.0;
            double out = 0.0;
            if (io->frost_table[c] > io->zwt_perched[c]) {
                const double q_perch_max = P->perched_baseflow_scalar * std::sin(io->topo_slope[c] * (RPI / 180.0));
                double wtsub = 0.0, q_perch = 0.0;
                for (int kk = k_perch; kk <= k_frost - 1; ++kk) {
                    q_perch = q_perch + k.hksat(kk) * k.dz(kk);
                    wtsub = wtsub + k.dz(kk);
                }
                if (wtsub > 0.0) q_perch = q_perch / wtsub;
                out = q_perch_max * q_perch * (io->frost_table[c] - io->zwt_perched[c]);
            }
            io->qflx_drain_perched[c] = io->qflx_drain_perched[c] + out;
            double drainage_tot = io->qflx_drain_perched[c] * dtime;
            for (int kk = k_perch; kk <= k_frost - 1; ++kk) {
                double s_y = k.watsat(kk) * (1. - o_pow(1. + 1.e3 * io->zwt_perched[c] / k.sucsat(kk), -1. / k.bsw(kk)));
                s_y = std::max(s_y, P->aq_sp_yield_min);
                double dl;
                if (kk == k_perch) dl = std::min(drainage_tot, (s_y * (k.zi(kk) - io->zwt_perched[c]) * 1.e3));
                else dl = std::min(drainage_tot, (s_y * (k.dz(kk)) * 1.e3));
                dl = std::max(dl, 0.0);
                drainage_tot = drainage_tot - dl;
                k.liq(kk) = k.liq(kk) - dl;
            }
            io->qflx_drain_perched[c] = io->qflx_drain_perched[c] - drainage_tot / dtime;
        } else {                               // SubsurfaceLateralFlow
            const int nb = io->nbedrock[c];
            double dzmm[NLEVSOI + 1];
            for (int j = 1; j <= NLEVSOI; ++j) {
                dzmm[j] = k.dz(j) * 1.e3;
                const double vol_ice = std::min(k.watsat(j), k.ice(j) / (k.dz(j) * DENICE));
                k.icefrac(j) = std::min(1.0, vol_ice / k.watsat(j));
            }
            io->qflx_drain[c] = 0.0;
            io->qflx_rsub_sat[c] = 0.0;
            double drainage = 0.0;
            io->qflx_latflow_in[c] = 0.0;
            io->qflx_latflow_out[c] = 0.0;
            int jwt = NLEVSOI;
            for (int j = 1; j <= NLEVSOI; ++j)
                if (io->zwt[c] <= k.zi(j)) { jwt = j - 1; break; }
            double dzsum = 0.0, icefracsum = 0.0;
            for (int j = std::max(jwt, 1); j <= NLEVSOI; ++j) {
                dzsum = dzsum + dzmm[j];
                icefracsum = icefracsum + k.icefrac(j) * dzmm[j];
            }
            const double ice_imped_col = o_pow(10.0, -P->e_ice * (icefracsum / dzsum));
            if (io->zwt[c] <= k.zi(nb))
                io->qflx_latflow_out[c] = ice_imped_col * P->baseflow_scalar * std::tan(RPI / 180.0 * io->topo_slope[c]) *
                                          o_pow(k.zi(nb) - io->zwt[c], P->n_baseflow);
            const double net = io->qflx_latflow_out[c] - io->qflx_latflow_in[c];
            if (io->zwt[c] <= k.zi(nb)) drainage = net;
            else drainage = 0.0;
            double drainage_tot = -drainage * dtime;
            if (drainage_tot > 0.) {
                for (int j = jwt + 1; j >= 1; --j) {
                    if (k.zi(j) < io->frost_table[c]) {
                        double s_y = k.watsat(j) * (1. - o_pow(1. + 1.e3 * io->zwt[c] / k.sucsat(j), -1. / k.bsw(j)));
                        s_y = std::max(s_y, P->aq_sp_yield_min);
                        double dl = std::min(drainage_tot, (s_y * k.dz(j) * 1.e3));
                        dl = std::max(dl, 0.0);
                        k.liq(j) = k.liq(j) + dl;
                        drainage_tot = drainage_tot - dl;
                        if (drainage_tot <= 0.) {
                            io->zwt[c] = io->zwt[c] - dl / s_y / 1000.0;
                            break;
                        } else {
                            io->zwt[c] = k.zi(j - 1);
                        }
                    }
                }
                io->h2osfc[c] = io->h2osfc[c] + drainage_tot;
            } else {
                for (int j = jwt + 1; j <= nb; ++j) {
                    double s_y = k.watsat(j) * (1. - o_pow(1. + 1.e3 * io->zwt[c] / k.sucsat(j), -1. / k.bsw(j)));
                    s_y = std::max(s_y, P->aq_sp_yield_min);
                    double dl = std::max(drainage_tot, -(s_y * (k.zi(j) - io->zwt[c]) * 1.e3));
                    dl = std::min(dl, 0.0);
                    k.liq(j) = k.liq(j) + dl;
                    drainage_tot = drainage_tot - dl;
                    if (drainage_tot >= 0.) {
                        io->zwt[c] = io->zwt[c] - dl / s_y / 1000.0;
                        break;
                    } else {
                        io->zwt[c] = k.zi(j);
                    }
                }
                drainage = drainage + drainage_tot / dtime;
            }
            io->zwt[c] = std::max(0.0, io->zwt[c]);
            io->zwt[c] = std::min(80.0, io->zwt[c]);
            for (int j = NLEVSOI; j >= 2; --j) {
                const double xsi = std::max(k.liq(j) - k.eff(j) * dzmm[j], 0.0);
                k.liq(j) = std::min(k.eff(j) * dzmm[j], k.liq(j));
                k.liq(j - 1) = k.liq(j - 1) + xsi;
            }
            double xs1 = std::max(std::max(k.liq(1) - WATMIN, 0.0) -
                                  std::max(0.0, (PONDMX + k.watsat(1) * dzmm[1] - k.ice(1) - WATMIN)), 0.0);
            k.liq(1) = k.liq(1) - xs1;
            io->h2osfc[c] = io->h2osfc[c] + xs1;
            io->qflx_rsub_sat[c] = 0.0;
            xs1 = std::max(std::max(k.ice(1), 0.0) - std::max(0.0, (PONDMX + k.watsat(1) * dzmm[1] - k.liq(1))), 0.0);
            k.ice(1) = std::min(std::max(0.0, PONDMX + k.watsat(1) * dzmm[1] - k.liq(1)), k.ice(1));
            io->qflx_ice_runoff_xs[c] = xs1 / dtime;
            for (int j = 1; j <= NLEVSOI - 1; ++j) {
                double xs;
                if (k.liq(j) < WATMIN) {
                    xs = WATMIN - k.liq(j);
                    if (j == jwt) io->zwt[c] = io->zwt[c] + xs / k.eff(j) / 1000.0;
                } else {
                    xs = 0.0;
                }
                k.liq(j) = k.liq(j) + xs;
                k.liq(j + 1) = k.liq(j + 1) - xs;
            }
            {
                const int j = NLEVSOI;
                double xs;
                if (k.liq(j) < WATMIN) {
                    xs = WATMIN - k.liq(j);
                    for (int i = NLEVSOI - 1; i >= 1; --i) {
                        const double avail = std::max(k.liq(i) - WATMIN - xs, 0.0);
                        if (avail >= xs) {
                            k.liq(j) = k.liq(j) + xs;
                            k.liq(i) = k.liq(i) - xs;
                            xs = 0.0;
                            break;
                        } else {
                            k.liq(j) = k.liq(j) + avail;
                            k.liq(i) = k.liq(i) - avail;
                            xs = xs - avail;
                        }
                    }
                } else {
                    xs = 0.0;
                }
                k.liq(j) = k.liq(j) + xs;
                io->qflx_rsub_sat[c] = io->qflx_rsub_sat[c] - xs / dtime;
            }
            io->qflx_drain[c] = io->qflx_rsub_sat[c] + drainage;
            io->qflx_qrgwl[c] = io->qflx_snwcp_liq[c];
        }
    }
    return 0;
}
