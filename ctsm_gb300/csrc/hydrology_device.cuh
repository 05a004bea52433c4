// hydrology_device.cuh -- per-column device forms of the water-table and
// drainage routines of the default hydrology (no aquifer layer, natural soil
// columns outside hillslopes), shared by the drop-in kernels and the
// resident step.  Each follows its reference routine statement by statement;
// default-real literals of the reference (sat_lev = 0.9) are reproduced as
// the single-precision values the Fortran compiler stores.
#pragma once
#include <cuda_runtime.h>
#include "ctsm_gpu.h"
#include "ctsm_device.cuh"
#include "soil_math.cuh"

namespace ctsmg {
namespace hydro {

constexpr double WATMIN = 0.01;          // clm_varcon.F90:81
constexpr double PONDMX = 0.0;           // clm_varcon.F90:116
constexpr double RPI = 3.14159265358979323846;
constexpr double AQUIFER_WATER_BASELINE = 5000.0;   // clm_varcon.F90:124

struct View {
    const ctsmg_hydrology_io& io;
    int c, ld;
    __device__ __forceinline__ size_t ss(int j) const { return c + (size_t)(j - LS) * ld; }
    __device__ __forceinline__ size_t g(int j) const { return c + (size_t)(j - 1) * ld; }
    __device__ __forceinline__ double zi(int j) const { return io.zi[c + (size_t)(j + NLEVSNO) * ld]; }
    __device__ __forceinline__ double vol(int k) const {
        return io.h2osoi_liq[ss(k)] / (io.dz[ss(k)] * DENH2O) + io.h2osoi_ice[ss(k)] / (io.dz[ss(k)] * DENICE);
    }
};

// std::max / std::min semantics, as the oracle evaluates the reference's max / min
__device__ __forceinline__ double mx(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double mn(double a, double b) { return (b < a) ? b : a; }

// ComputeFsatTopmodel + SaturatedExcessRunoff (SaturatedExcessRunoffMod.F90:200-360)
__device__ __forceinline__ void saturated_excess_runoff(const ctsmg_hydrology_io& io, int c, double fff) {
    const double zt = (io.frost_table[c] > io.zwt_perched[c] && io.frost_table[c] <= io.zwt[c]) ? io.zwt_perched[c]
                                                                                                 : io.zwt[c];
    const double fsat = io.wtfact[c] * fm::exp(-0.5 * fff * zt);
    io.fsat[c] = fsat;
    io.qflx_sat_excess_surf[c] = fsat * io.qflx_rain_plus_snomelt[c];
    io.fcov[c] = fsat;
}

// SetQflxInputs (SoilHydrologyMod.F90:298-366), InfiltrationExcessRunoff with
// the hksat qinmax (InfiltrationExcessRunoffMod.F90:196-304),
// RouteInfiltrationExcess (:369-423, soil columns), UpdateH2osfc with
// QflxH2osfcSurf / QflxH2osfcDrain and truncate_small_values
// (SurfaceWaterMod.F90:345-556, NumericsMod.F90:50-99) and Infiltration
// (:426-457): the infiltration SoilWater takes as input.
__device__ __forceinline__ void infiltration_chain(const ctsmg_hydrology_io& io, int c,
                                                   const ctsmg_soilhydrology_params& P, double dtime) {
    const View v{io, c, io.ldc};
    const double fh = io.frac_h2osfc[c];
    // SetQflxInputs
    const double top = io.qflx_rain_plus_snomelt[c] + io.qflx_snow_h2osfc[c] + io.qflx_floodc[c];
    double fsno, qflx_evap;
    if (io.snl[c] >= 0) { fsno = 0.0; qflx_evap = io.qflx_liqevap_from_top_layer_col[c]; }
    else { fsno = io.frac_sno_eff[c]; qflx_evap = io.qflx_ev_soil_col[c]; }
    double in_soil = (1.0 - fh) * (top - io.qflx_sat_excess_surf[c]);
    double to_h2osfc = fh * (top - io.qflx_sat_excess_surf[c]);
    in_soil = in_soil - (1.0 - fsno - fh) * qflx_evap;
    to_h2osfc = to_h2osfc - fh * io.qflx_ev_h2osfc_col[c];
    io.qflx_top_soil[c] = top;
    io.qflx_in_soil[c] = in_soil;
    io.qflx_top_soil_to_h2osfc[c] = to_h2osfc;
    // InfiltrationExcessRunoff (minval over levels 1..3 of 10^(-e_ice icefrac) hksat)
    double qmu = pow10_dd(-P.e_ice * (io.icefrac[v.g(1)])) * io.hksat[v.g(1)];
#pragma unroll
    for (int j = 2; j <= 3; ++j) {
        const double q = pow10_dd(-P.e_ice * (io.icefrac[v.g(j)])) * io.hksat[v.g(j)];
        qmu = (q < qmu) ? q : qmu;
    }
    const double qinmax = (1.0 - io.fsat[c]) * qmu;
    const double infl_excess = mx(0.0, (in_soil - (1.0 - fh) * qinmax));
    io.qinmax[c] = qinmax;
    io.qflx_infl_excess[c] = infl_excess;
    // RouteInfiltrationExcess
    const double limited = in_soil - infl_excess;
    double in_h2osfc, excess_surf;
    if (P.h2osfcflag != 0) { in_h2osfc = to_h2osfc + infl_excess; excess_surf = 0.0; }
    else { in_h2osfc = to_h2osfc; excess_surf = infl_excess; }
    io.qflx_in_soil_limited[c] = limited;
    io.qflx_in_h2osfc[c] = in_h2osfc;
    io.qflx_infl_excess_surf[c] = excess_surf;
    // UpdateH2osfc
    const double h0 = io.h2osfc[c], thr = io.h2osfc_thresh[c];
    double frac_infclust = 0.0;
    if (P.h2osfcflag == 1) {
        const double fn = io.frac_h2osfc_nosnow[c];
        frac_infclust = (fn <= P.pc) ? 0.0 : fm::pow(fn - P.pc, P.mu);
    }
    double surf;
    if (h0 > thr && P.h2osfcflag != 0) {
        const double k_wet = 1.0e-4 * sin((RPI / 180.0) * io.topo_slope[c]);
        surf = k_wet * frac_infclust * (h0 - thr);
        surf = mn(surf, (h0 - thr) / dtime);
    } else {
        surf = 0.0;
    }
    if (surf < (double)1.0e-8f) surf = 0.0;
    io.qflx_h2osfc_surf[c] = surf;
    double hp = h0 + (in_h2osfc - surf) * dtime;
    if (fabs(hp) < 1.e-13 * fabs(h0)) hp = 0.0;
    double drain;
    if (hp < 0.0) {
        drain = hp / dtime;
    } else {
        drain = mn(fh * qinmax, hp / dtime);
        if (P.h2osfcflag == 0) drain = mx(0.0, hp / dtime);
    }
    io.qflx_h2osfc_drain[c] = drain;
    double h1 = hp - drain * dtime;
    if (fabs(h1) < 1.e-13 * fabs(hp)) h1 = 0.0;
    io.h2osfc[c] = h1;
    // Infiltration
    io.qflx_infl[c] = limited + drain;
}

// PerchedWaterTable (SoilHydrologyMod.F90:1525-1641)
__device__ __forceinline__ void perched_water_table(const ctsmg_hydrology_io& io, int c) {
    const View v{io, c, io.ldc};
    const double sat_lev = (double)0.9f;
    int k_frz = (io.t_soisno[v.ss(1)] > TFRZ) ? NLEVSOI : 1;
#pragma unroll 1
    for (int k = 2; k <= NLEVSOI; ++k)
        if (io.t_soisno[v.ss(k - 1)] > TFRZ && io.t_soisno[v.ss(k)] <= TFRZ) { k_frz = k; break; }
    const double ft = v.zi(k_frz - 1);
    io.frost_table[c] = ft;
    io.zwt_perched[c] = ft;
    if (io.zwt[c] < ft && io.t_soisno[v.ss(k_frz)] <= TFRZ) {
        // water table above the frost table: nothing perches
    } else if (k_frz > 1) {
        int k_perch = 1;
#pragma unroll 1
        for (int k = k_frz; k >= 1; --k) {
            const double hv = v.vol(k);
            io.h2osoi_vol[v.g(k)] = hv;
            if (hv / io.watsat[v.g(k)] <= sat_lev) { k_perch = k; break; }
        }
        if (io.t_soisno[v.ss(k_frz)] > TFRZ) k_perch = k_frz;
        if (k_frz > k_perch) {
            const double s1 = v.vol(k_perch) / io.watsat[v.g(k_perch)];
            const double s2 = v.vol(k_perch + 1) / io.watsat[v.g(k_perch + 1)];
            if (s1 > s2) {
                io.zwt_perched[c] = v.zi(k_perch - 1);
            } else {
                const double m = (io.z[v.ss(k_perch + 1)] - io.z[v.ss(k_perch)]) / (s2 - s1);
                const double b = io.z[v.ss(k_perch + 1)] - m * s2;
                io.zwt_perched[c] = mx(0.0, m * sat_lev + b);
            }
        }
    }
}

// ThetaBasedWaterTable (SoilHydrologyMod.F90:1933-2025)
__device__ __forceinline__ void theta_based_water_table(const ctsmg_hydrology_io& io, int c) {
    const View v{io, c, io.ldc};
    const double sat_lev = (double)0.9f;
    const int nb = io.nbedrock[c];
    int k_zwt = nb;
    bool sat = true;
#pragma unroll 1
    for (int k = nb; k >= 1; --k) {
        const double hv = v.vol(k);
        io.h2osoi_vol[v.g(k)] = hv;
        if (hv / io.watsat[v.g(k)] <= sat_lev) { k_zwt = k; sat = false; break; }
    }
    if (sat) k_zwt = 1;
    double zwt;
    if (k_zwt == 1) {
        zwt = v.zi(1);
    } else if (k_zwt < nb) {
        const double s1 = v.vol(k_zwt) / io.watsat[v.g(k_zwt)];
        const double s2 = v.vol(k_zwt + 1) / io.watsat[v.g(k_zwt + 1)];
        const double m = (io.z[v.ss(k_zwt + 1)] - io.z[v.ss(k_zwt)]) / (s2 - s1);
        const double b = io.z[v.ss(k_zwt + 1)] - m * s2;
        zwt = mx(0.0, m * sat_lev + b);
    } else {
        zwt = v.zi(nb);
    }
    io.zwt[c] = zwt;
}

__device__ __forceinline__ double specific_yield(const ctsmg_hydrology_io& io, const View& v, int k, double depth,
                                                 double aq_sp_yield_min) {
    const double s_y = io.watsat[v.g(k)] *
                       (1.0 - fm::pow(1.0 + 1.e3 * depth / io.sucsat[v.g(k)], -1.0 / io.bsw[v.g(k)]));
    return mx(s_y, aq_sp_yield_min);
}

// PerchedLateralFlow (SoilHydrologyMod.F90:1645-1929), non-hillslope columns
__device__ __forceinline__ void perched_lateral_flow(const ctsmg_hydrology_io& io, int c,
                                                     const ctsmg_soilhydrology_params& P, double dtime) {
    const View v{io, c, io.ldc};
    const int nb = io.nbedrock[c];
    const double ft = io.frost_table[c], zp = io.zwt_perched[c];
    int k_frost = nb, k_perch = nb;
#pragma unroll 1
    for (int k = 1; k <= nb; ++k)
        if (ft >= v.zi(k - 1) && ft < v.zi(k)) { k_frost = k; break; }
#pragma unroll 1
    for (int k = 1; k <= nb; ++k)
        if (zp >= v.zi(k - 1) && zp < v.zi(k)) { k_perch = k; break; }
    double out = 0.0;
    if (ft > zp) {
        const double q_perch_max = P.perched_baseflow_scalar * sin(io.topo_slope[c] * (RPI / 180.0));
        double wtsub = 0.0, q_perch = 0.0;
#pragma unroll 1
        for (int k = k_perch; k <= k_frost - 1; ++k) {
            q_perch = q_perch + io.hksat[v.g(k)] * io.dz[v.ss(k)];
            wtsub = wtsub + io.dz[v.ss(k)];
        }
        if (wtsub > 0.0) q_perch = q_perch / wtsub;
        out = q_perch_max * q_perch * (ft - zp);
    }
    double drain = 0.0 + out;
    double drainage_tot = drain * dtime;
#pragma unroll 1
    for (int k = k_perch; k <= k_frost - 1; ++k) {
        const double s_y = specific_yield(io, v, k, zp, P.aq_sp_yield_min);
        double dl = (k == k_perch) ? mn(drainage_tot, (s_y * (v.zi(k) - zp) * 1.e3))
                                   : mn(drainage_tot, (s_y * (io.dz[v.ss(k)]) * 1.e3));
        dl = mx(dl, 0.0);
        drainage_tot = drainage_tot - dl;
        io.h2osoi_liq[v.ss(k)] = io.h2osoi_liq[v.ss(k)] - dl;
    }
    io.qflx_drain_perched[c] = drain - drainage_tot / dtime;
}

// SubsurfaceLateralFlow (SoilHydrologyMod.F90:2029-2565), non-hillslope
// natural soil columns
__device__ __forceinline__ void subsurface_lateral_flow(const ctsmg_hydrology_io& io, int c,
                                                        const ctsmg_soilhydrology_params& P, double dtime) {
    const View v{io, c, io.ldc};
    const int nb = io.nbedrock[c];
    double* liq = io.h2osoi_liq;
    double* ice = io.h2osoi_ice;
#pragma unroll 1
    for (int j = 1; j <= NLEVSOI; ++j) {
        const double ws = io.watsat[v.g(j)];
        const double q = ice[v.ss(j)] / (io.dz[v.ss(j)] * DENICE);
        const double vol_ice = mn(ws, q);
        io.icefrac[v.g(j)] = mn(1.0, vol_ice / ws);
    }
    double zwt = io.zwt[c];
    int jwt = NLEVSOI;
#pragma unroll 1
    for (int j = 1; j <= NLEVSOI; ++j)
        if (zwt <= v.zi(j)) { jwt = j - 1; break; }
    double dzsum = 0.0, icefracsum = 0.0;
#pragma unroll 1
    for (int j = (jwt > 1 ? jwt : 1); j <= NLEVSOI; ++j) {
        const double dzmm = io.dz[v.ss(j)] * 1.e3;
        dzsum = dzsum + dzmm;
        icefracsum = icefracsum + io.icefrac[v.g(j)] * dzmm;
    }
    const double ice_imped_col = pow10_dd(-P.e_ice * (icefracsum / dzsum));
    double latflow_out = 0.0;
    const double zib = v.zi(nb);
    if (zwt <= zib)
        latflow_out = ice_imped_col * P.baseflow_scalar * tan(RPI / 180.0 * io.topo_slope[c]) * fm::pow(zib - zwt, P.n_baseflow);
    io.qflx_latflow_out[c] = latflow_out;
    io.qflx_latflow_in[c] = 0.0;
    const double net = latflow_out - 0.0;
    double drainage = (zwt <= zib) ? net : 0.0;
    double drainage_tot = -drainage * dtime;
    if (drainage_tot > 0.0) {                       // rising water table
        const double ft = io.frost_table[c];
#pragma unroll 1
        for (int j = jwt + 1; j >= 1; --j) {
            if (v.zi(j) < ft) {
                const double s_y = specific_yield(io, v, j, zwt, P.aq_sp_yield_min);
                double dl = mn(drainage_tot, (s_y * io.dz[v.ss(j)] * 1.e3));
                dl = mx(dl, 0.0);
                liq[v.ss(j)] = liq[v.ss(j)] + dl;
                drainage_tot = drainage_tot - dl;
                if (drainage_tot <= 0.0) { zwt = zwt - dl / s_y / 1000.0; break; }
                zwt = v.zi(j - 1);
            }
        }
        io.h2osfc[c] = io.h2osfc[c] + drainage_tot;
    } else {                                        // deepening water table
#pragma unroll 1
        for (int j = jwt + 1; j <= nb; ++j) {
            const double s_y = specific_yield(io, v, j, zwt, P.aq_sp_yield_min);
            double dl = mx(drainage_tot, -(s_y * (v.zi(j) - zwt) * 1.e3));
            dl = mn(dl, 0.0);
            liq[v.ss(j)] = liq[v.ss(j)] + dl;
            drainage_tot = drainage_tot - dl;
            if (drainage_tot >= 0.0) { zwt = zwt - dl / s_y / 1000.0; break; }
            zwt = v.zi(j);
        }
        drainage = drainage + drainage_tot / dtime;
    }
    zwt = mx(0.0, zwt);
    zwt = mn(80.0, zwt);
    // excess above saturation moves up; the top layer's goes to h2osfc
#pragma unroll 1
    for (int j = NLEVSOI; j >= 2; --j) {
        const double cap = io.eff_porosity[v.g(j)] * (io.dz[v.ss(j)] * 1.e3);
        const double xsi = mx(liq[v.ss(j)] - cap, 0.0);
        liq[v.ss(j)] = mn(cap, liq[v.ss(j)]);
        liq[v.ss(j - 1)] = liq[v.ss(j - 1)] + xsi;
    }
    const double dz1mm = io.dz[v.ss(1)] * 1.e3, ws1 = io.watsat[v.g(1)];
    double xs1 = mx(mx(liq[v.ss(1)] - WATMIN, 0.0) - mx(0.0, (PONDMX + ws1 * dz1mm - ice[v.ss(1)] - WATMIN)), 0.0);
    liq[v.ss(1)] = liq[v.ss(1)] - xs1;
    io.h2osfc[c] = io.h2osfc[c] + xs1;
    double rsub_sat = 0.0;
    xs1 = mx(mx(ice[v.ss(1)], 0.0) - mx(0.0, (PONDMX + ws1 * dz1mm - liq[v.ss(1)])), 0.0);
    ice[v.ss(1)] = mn(mx(0.0, PONDMX + ws1 * dz1mm - liq[v.ss(1)]), ice[v.ss(1)]);
    io.qflx_ice_runoff_xs[c] = xs1 / dtime;
    // liquid below watmin is borrowed from the layer below
#pragma unroll 1
    for (int j = 1; j <= NLEVSOI - 1; ++j) {
        double xs = 0.0;
        if (liq[v.ss(j)] < WATMIN) {
            xs = WATMIN - liq[v.ss(j)];
            if (j == jwt) zwt = zwt + xs / io.eff_porosity[v.g(j)] / 1000.0;
        }
        liq[v.ss(j)] = liq[v.ss(j)] + xs;
        liq[v.ss(j + 1)] = liq[v.ss(j + 1)] - xs;
    }
    {
        const int j = NLEVSOI;
        double xs = 0.0;
        if (liq[v.ss(j)] < WATMIN) {
            xs = WATMIN - liq[v.ss(j)];
#pragma unroll 1
            for (int i = NLEVSOI - 1; i >= 1; --i) {
                const double avail = mx(liq[v.ss(i)] - WATMIN - xs, 0.0);
                if (avail >= xs) {
                    liq[v.ss(j)] = liq[v.ss(j)] + xs;
                    liq[v.ss(i)] = liq[v.ss(i)] - xs;
                    xs = 0.0;
                    break;
                }
                liq[v.ss(j)] = liq[v.ss(j)] + avail;
                liq[v.ss(i)] = liq[v.ss(i)] - avail;
                xs = xs - avail;
            }
        }
        liq[v.ss(j)] = liq[v.ss(j)] + xs;
        rsub_sat = rsub_sat - xs / dtime;
    }
    io.zwt[c] = zwt;
    io.qflx_rsub_sat[c] = rsub_sat;
    io.qflx_drain[c] = rsub_sat + drainage;
    io.qflx_qrgwl[c] = io.qflx_snwcp_liq[c];
}

__device__ __forceinline__ int water_table_index(const View& v, double zwt) {
    int jwt = NLEVSOI;
#pragma unroll 1
    for (int j = 1; j <= NLEVSOI; ++j)
        if (zwt <= v.zi(j)) { jwt = j - 1; break; }
    return jwt;
}

// The perched water table of the aquifer-layer path (frost table at the
// node depth z(k_frz), SoilHydrologyMod.F90:782-856 and 932-995); returns
// k_frz and k_perch, and whether the water table is above the frost table.
struct Perch { int k_frz, k_perch; bool wt_above; };
__device__ __forceinline__ Perch aquifer_perched(const ctsmg_hydrology_io& io, const View& v, int c, bool write_vol) {
    const double sat_lev = (double)0.9f;
    Perch r{};
    r.k_frz = (io.t_soisno[v.ss(1)] > TFRZ) ? NLEVSOI : 1;
#pragma unroll 1
    for (int k = 2; k <= NLEVSOI; ++k)
        if (io.t_soisno[v.ss(k - 1)] > TFRZ && io.t_soisno[v.ss(k)] <= TFRZ) { r.k_frz = k; break; }
    const double ft = io.z[v.ss(r.k_frz)];
    io.frost_table[c] = ft;
    io.zwt_perched[c] = ft;
    r.wt_above = io.zwt[c] < ft && io.t_soisno[v.ss(r.k_frz)] <= TFRZ;
    r.k_perch = 1;
    if (r.wt_above) return r;
#pragma unroll 1
    for (int k = r.k_frz; k >= 1; --k) {
        const double hv = v.vol(k);
        if (write_vol) io.h2osoi_vol[v.g(k)] = hv;
        if (hv / io.watsat[v.g(k)] <= sat_lev) { r.k_perch = k; break; }
    }
    if (io.t_soisno[v.ss(r.k_frz)] > TFRZ) r.k_perch = r.k_frz;
    if (r.k_frz > r.k_perch) {
        const double s1 = v.vol(r.k_perch) / io.watsat[v.g(r.k_perch)];
        const double s2 = v.vol(r.k_perch + 1) / io.watsat[v.g(r.k_perch + 1)];
        const double m = (io.z[v.ss(r.k_perch + 1)] - io.z[v.ss(r.k_perch)]) / (s2 - s1);
        const double b = io.z[v.ss(r.k_perch + 1)] - m * s2;
        io.zwt_perched[c] = mx(0.0, m * sat_lev + b);
    }
    return r;
}

// WaterTable (SoilHydrologyMod.F90:607-861)
__device__ __forceinline__ void water_table(const ctsmg_hydrology_io& io, int c, const ctsmg_soilhydrology_params& P,
                                            double dtime) {
    const View v{io, c, io.ldc};
    io.qflx_drain[c] = 0.0;
    io.qflx_rsub_sat[c] = 0.0;
    io.qflx_drain_perched[c] = 0.0;
    double zwt = io.zwt[c];
    const int jwt = water_table_index(v, zwt);
    double rous = specific_yield(io, v, NLEVSOI, zwt, P.aq_sp_yield_min);
    const double qcharge = io.qcharge[c];
    if (jwt == NLEVSOI) {
        io.wa[c] = io.wa[c] + qcharge * dtime;
        zwt = zwt - (qcharge * dtime) / 1000.0 / rous;
    } else {
        double tot = qcharge * dtime;
        if (tot > 0.0) {                                  // rising water table
#pragma unroll 1
            for (int j = jwt + 1; j >= 1; --j) {
                const double s_y = specific_yield(io, v, j, zwt, P.aq_sp_yield_min);
                double layer = mn(tot, (s_y * (zwt - v.zi(j - 1)) * 1.e3));
                layer = mx(layer, 0.0);
                if (s_y > 0.0) zwt = zwt - layer / s_y / 1000.0;
                tot = tot - layer;
                if (tot <= 0.0) break;
            }
        } else {                                          // deepening water table
#pragma unroll 1
            for (int j = jwt + 1; j <= NLEVSOI; ++j) {
                const double s_y = specific_yield(io, v, j, zwt, P.aq_sp_yield_min);
                double layer = mx(tot, -(s_y * (v.zi(j) - zwt) * 1.e3));
                layer = mn(layer, 0.0);
                tot = tot - layer;
                if (tot >= 0.0) { zwt = zwt - layer / s_y / 1000.0; break; }
                zwt = v.zi(j);
            }
            if (tot > 0.0) zwt = zwt - tot / 1000.0 / rous;
        }
    }
    io.zwt[c] = zwt;
    aquifer_perched(io, v, c, true);
}

// Drainage (SoilHydrologyMod.F90:864-1410), non-VIC natural soil columns
__device__ __forceinline__ void drainage(const ctsmg_hydrology_io& io, int c, const ctsmg_soilhydrology_params& P,
                                         double dtime) {
    const View v{io, c, io.ldc};
    double* liq = io.h2osoi_liq;
    double* ice = io.h2osoi_ice;
#pragma unroll 1
    for (int j = 1; j <= NLEVSOI; ++j) {
        const double ws = io.watsat[v.g(j)];
        const double vol_ice = mn(ws, ice[v.ss(j)] / (io.dz[v.ss(j)] * DENICE));
        io.icefrac[v.g(j)] = mn(1.0, vol_ice / ws);
    }
    double rsub_sat = 0.0, rsub_top = 0.0;
    double zwt = io.zwt[c];
    int jwt = water_table_index(v, zwt);
    const double q_perch_max = P.perched_baseflow_scalar * sin(io.topo_slope[c] * (RPI / 180.0));
    const Perch pr = aquifer_perched(io, v, c, false);
    const double ft = io.frost_table[c];
    double drain_perched = 0.0;
    auto imped_k = [&](int k) {
        const int k1 = (NLEVSOI < k + 1) ? NLEVSOI : k + 1;
        return pow10_dd(-P.e_ice * (0.5 * (io.icefrac[v.g(k)] + io.icefrac[v.g(k1)])));
    };
    if (pr.wt_above) {
        double wtsub = 0.0, q_perch = 0.0;
#pragma unroll 1
        for (int k = jwt + 1; k <= pr.k_frz; ++k) {
            const double dzmm = io.dz[v.ss(k)] * 1.e3;
            q_perch = q_perch + imped_k(k) * io.hksat[v.g(k)] * dzmm;
            wtsub = wtsub + dzmm;
        }
        if (wtsub > 0.0) q_perch = q_perch / wtsub;
        drain_perched = q_perch_max * q_perch * (ft - zwt);
        double tot = -drain_perched * dtime;
#pragma unroll 1
        for (int k = jwt + 1; k <= pr.k_frz; ++k) {
            double layer = mx(tot, -(liq[v.ss(k)] - WATMIN));
            layer = mn(layer, 0.0);
            tot = tot - layer;
            liq[v.ss(k)] = liq[v.ss(k)] + layer;
            if (tot >= 0.0) { zwt = zwt - layer / io.eff_porosity[v.g(k)] / 1000.0; break; }
            zwt = v.zi(k);
        }
        drain_perched = drain_perched + tot / dtime;
        jwt = water_table_index(v, zwt);
    } else {
        if (pr.k_frz > pr.k_perch) {
            double wtsub = 0.0, q_perch = 0.0;
#pragma unroll 1
            for (int k = pr.k_perch; k <= pr.k_frz; ++k) {
                const double dzmm = io.dz[v.ss(k)] * 1.e3;
                q_perch = q_perch + imped_k(k) * io.hksat[v.g(k)] * dzmm;
                wtsub = wtsub + dzmm;
            }
            if (wtsub > 0.0) q_perch = q_perch / wtsub;
            double zp = io.zwt_perched[c];
            drain_perched = q_perch_max * q_perch * (ft - zp);
            double tot = -drain_perched * dtime;
#pragma unroll 1
            for (int k = pr.k_perch + 1; k <= pr.k_frz; ++k) {
                double layer = mx(tot, -(liq[v.ss(k)] - WATMIN));
                layer = mn(layer, 0.0);
                tot = tot - layer;
                liq[v.ss(k)] = liq[v.ss(k)] + layer;
                if (tot >= 0.0) { zp = zp - layer / io.eff_porosity[v.g(k)] / 1000.0; break; }
                zp = v.zi(k);
            }
            io.zwt_perched[c] = zp;
            drain_perched = drain_perched + tot / dtime;
        } else {
            drain_perched = 0.0;
        }
        const double fff = 1.0 / io.hkdepth[c];
        double dzsum = 0.0, icefracsum = 0.0;
#pragma unroll 1
        for (int j = (jwt > 1 ? jwt : 1); j <= NLEVSOI; ++j) {
            const double dzmm = io.dz[v.ss(j)] * 1.e3;
            dzsum = dzsum + dzmm;
            icefracsum = icefracsum + io.icefrac[v.g(j)] * dzmm;
        }
        const double imped = pow10_dd(-P.e_ice * (icefracsum / dzsum));
        const double rsub_top_max = 10.0 * sin((RPI / 180.0) * io.topo_slope[c]);
        rsub_top = imped * rsub_top_max * fm::exp(-fff * zwt);
        const double rous = specific_yield(io, v, NLEVSOI, zwt, P.aq_sp_yield_min);
        if (jwt == NLEVSOI) {
            double wa = io.wa[c] - rsub_top * dtime;
            zwt = zwt + (rsub_top * dtime) / 1000.0 / rous;
            liq[v.ss(NLEVSOI)] = liq[v.ss(NLEVSOI)] + mx(0.0, (wa - AQUIFER_WATER_BASELINE));
            io.wa[c] = mn(wa, AQUIFER_WATER_BASELINE);
        } else {
            double tot = -rsub_top * dtime;
            // tot > 0 cannot happen here (rsub_top >= 0); the reference stops the run on it
#pragma unroll 1
            for (int j = jwt + 1; j <= NLEVSOI; ++j) {
                const double s_y = specific_yield(io, v, j, zwt, P.aq_sp_yield_min);
                double layer = mx(tot, -(s_y * (v.zi(j) - zwt) * 1.e3));
                layer = mn(layer, 0.0);
                liq[v.ss(j)] = liq[v.ss(j)] + layer;
                tot = tot - layer;
                if (tot >= 0.0) { zwt = zwt - layer / s_y / 1000.0; break; }
                zwt = v.zi(j);
            }
            zwt = zwt - tot / 1000.0 / rous;
            io.wa[c] = io.wa[c] + tot;
            jwt = water_table_index(v, zwt);
        }
        zwt = mx(0.0, zwt);
        zwt = mn(80.0, zwt);
    }
    io.qflx_drain_perched[c] = drain_perched;
    // excess above saturation moves up; the top layer's goes to h2osfc
#pragma unroll 1
    for (int j = NLEVSOI; j >= 2; --j) {
        const double cap = io.eff_porosity[v.g(j)] * (io.dz[v.ss(j)] * 1.e3);
        const double xsi = mx(liq[v.ss(j)] - cap, 0.0);
        liq[v.ss(j)] = mn(cap, liq[v.ss(j)]);
        liq[v.ss(j - 1)] = liq[v.ss(j - 1)] + xsi;
    }
    const double dz1mm = io.dz[v.ss(1)] * 1.e3, ws1 = io.watsat[v.g(1)];
    double xs1 = mx(mx(liq[v.ss(1)] - WATMIN, 0.0) - mx(0.0, (PONDMX + ws1 * dz1mm - ice[v.ss(1)] - WATMIN)), 0.0);
    liq[v.ss(1)] = liq[v.ss(1)] - xs1;
    if (P.h2osfcflag == 1) { io.h2osfc[c] = io.h2osfc[c] + xs1; rsub_sat = 0.0; }
    else rsub_sat = xs1 / dtime;
    xs1 = mx(mx(ice[v.ss(1)], 0.0) - mx(0.0, (PONDMX + ws1 * dz1mm - liq[v.ss(1)])), 0.0);
    ice[v.ss(1)] = mn(mx(0.0, PONDMX + ws1 * dz1mm - liq[v.ss(1)]), ice[v.ss(1)]);
    io.qflx_ice_runoff_xs[c] = xs1 / dtime;
#pragma unroll 1
    for (int j = 1; j <= NLEVSOI - 1; ++j) {
        double xs = 0.0;
        if (liq[v.ss(j)] < WATMIN) {
            xs = WATMIN - liq[v.ss(j)];
            if (j == jwt) zwt = zwt + xs / io.eff_porosity[v.g(j)] / 1000.0;
        }
        liq[v.ss(j)] = liq[v.ss(j)] + xs;
        liq[v.ss(j + 1)] = liq[v.ss(j + 1)] - xs;
    }
    {
        const int j = NLEVSOI;
        double xs = 0.0;
        if (liq[v.ss(j)] < WATMIN) {
            xs = WATMIN - liq[v.ss(j)];
#pragma unroll 1
            for (int i = NLEVSOI - 1; i >= 1; --i) {
                const double avail = mx(liq[v.ss(i)] - WATMIN - xs, 0.0);
                if (avail >= xs) {
                    liq[v.ss(j)] = liq[v.ss(j)] + xs;
                    liq[v.ss(i)] = liq[v.ss(i)] - xs;
                    xs = 0.0;
                    break;
                }
                liq[v.ss(j)] = liq[v.ss(j)] + avail;
                liq[v.ss(i)] = liq[v.ss(i)] - avail;
                xs = xs - avail;
            }
        }
        liq[v.ss(j)] = liq[v.ss(j)] + xs;
        rsub_top = rsub_top - xs / dtime;
    }
    io.zwt[c] = zwt;
    io.qflx_rsub_sat[c] = rsub_sat;
    io.qflx_drain[c] = rsub_sat + rsub_top;
    io.qflx_qrgwl[c] = io.qflx_snwcp_liq[c];
}

} // namespace hydro
} // namespace ctsmg
