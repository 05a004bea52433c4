// soilfluxes_device.cuh -- SoilFluxes for one natural-vegetation patch
// (src/biogeophys/SoilFluxesMod.F90:163-496), shared by the drop-in kernel and
// the fused model step.  gfortran evaluates x**3 and x**4 as x*x*x and
// (x*x)*(x*x); a*b/c as (a*b)/c.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "ctsm_gpu.h"
#include "ctsm_device.cuh"
#include "fastmath.cuh"

namespace ctsmg {
namespace sfx {
constexpr double HVAP_SF = 2.501e6;     // clm_varcon hvap (J/kg)
__device__ __forceinline__ double p3(double x) { return x * x * x; }
__device__ __forceinline__ double p4(double x) { const double x2 = x * x; return x2 * x2; }
} // namespace sfx

// Patch p (0-based) of column c (0-based position in the io arrays).
__device__ __forceinline__ void soilfluxes_patch(const ctsmg_soilfluxes_io& io, int p, int c, double dtime) {
    using sfx::p3;
    using sfx::p4;
    using sfx::HVAP_SF;
    const int ld = io.ldc, snl = io.snl[c], jtop = snl + 1;
    auto SS = [&](const double* a, int j) { return a[c + (size_t)(j - LS) * ld]; };
    const double fsno = io.frac_sno_eff[c], fh2o = io.frac_h2osfc[c], th2o_bef = io.t_h2osfc_bef[c];
    // ground temperature before the step and its increment (:168-185)
    double t_grnd0;
    if (snl < 0) t_grnd0 = fsno * SS(io.tssbef, jtop) + (1.0 - fsno - fh2o) * SS(io.tssbef, 1) + fh2o * th2o_bef;
    else t_grnd0 = (1.0 - fh2o) * SS(io.tssbef, 1) + fh2o * th2o_bef;
    const double tinc = io.t_grnd[c] - t_grnd0;
    // fluxes for the temperature increment (:189-205)
    double sh = io.eflx_sh_grnd[p] + tinc * io.cgrnds[p];
    double ev = io.qflx_evap_soi[p] + tinc * io.cgrndl[p];
    double ev_snow = io.qflx_ev_snow[p] + tinc * io.cgrndl[p];
    const double ev_soil = io.qflx_ev_soil[p] + tinc * io.cgrndl[p];
    const double ev_h2osfc = io.qflx_ev_h2osfc[p] + tinc * io.cgrndl[p];
    // evaporation and dew of the top layer (:215-250)
    const double liq = SS(io.h2osoi_liq, jtop), ice = SS(io.h2osoi_ice, jtop);
    double liqevap = 0.0, solidevap = 0.0, soliddew = 0.0, liqdew = 0.0;
    if (ev_snow >= 0.0) {
        liqevap = (liq + ice > 0.0) ? fmax(ev_snow * (liq / (liq + ice)), 0.0) : 0.0;
        solidevap = ev_snow - liqevap;
    } else if (io.t_grnd[c] < TFRZ) {
        soliddew = fabs(ev_snow);
    } else {
        liqdew = fabs(ev_snow);
    }
    // evaporation limits (:282-327)
    const double htvp = io.htvp[c];
    if (jtop < 1) {
        const double lim = (ice + liq) / (fsno * dtime);
        if (ev_snow > lim) {
            const double demand = ev_snow;
            ev_snow = lim;
            ev = ev - fsno * (demand - lim);
            liqevap = fmax(liq / (fsno * dtime), 0.0);
            solidevap = fmax(ice / (fsno * dtime), 0.0);
            sh = sh + fsno * (demand - lim) * htvp;
        }
    }
    if (jtop == 1 && fh2o < 1.0) {
        const double lim = ice / (dtime * (1.0 - fh2o));
        if (solidevap >= lim) {
            const double demand = solidevap;
            solidevap = lim;
            liqevap = liqevap + (demand - lim);
        }
    }
    // soil heat flux (:343-351)
    const double emg = io.emg[c], forc_lwrad = io.forc_lwrad[c];
    const double lw_grnd = (fsno * p4(SS(io.tssbef, jtop)) + (1.0 - fsno - fh2o) * p4(SS(io.tssbef, 1)) +
                            fh2o * p4(th2o_bef));
    const double fv = fm::i2d(1 - io.frac_veg_nosno[p]);
    const double esg = ((1.0 - fsno) * io.sabg_soil[p] + fsno * io.sabg_snow[p]) + io.dlrad[p] + fv * emg * forc_lwrad -
                       emg * SB * lw_grnd - emg * SB * p3(t_grnd0) * (4.0 * tinc) - (sh + ev * htvp);
    // totals and partitions (:375-393)
    const double evap_veg = io.qflx_evap_veg[p], tran = io.qflx_tran_veg[p];
    io.eflx_sh_tot[p] = io.eflx_sh_veg[p] + sh;
    io.qflx_evap_tot[p] = evap_veg + ev;
    io.eflx_lh_tot[p] = HVAP_SF * evap_veg + htvp * ev;
    io.qflx_evap_can[p] = evap_veg - tran;
    io.eflx_lh_vege[p] = (evap_veg - tran) * HVAP_SF;
    io.eflx_lh_vegt[p] = tran * HVAP_SF;
    io.eflx_lh_grnd[p] = ev * htvp;
    // soil energy error (:401-429)
    double err = esg - io.xmf[c] - io.xmf_h2osfc[c] - fh2o * (io.t_h2osfc[c] - th2o_bef) * (io.c_h2osfc[c] / dtime);
    err = err + io.eflx_h2osfc_to_snow[c];
#pragma unroll 1
    for (int j = jtop; j <= NLEVGRND; ++j) {
        const double dT = SS(io.t_soisno, j) - SS(io.tssbef, j);
        if (j < 1) err = err - fsno * dT / SS(io.fact, j);
        else err = err - dT / SS(io.fact, j);
    }
    // emitted longwave (:464-489)
    const double lwout = io.ulrad[p] + fv * (1.0 - emg) * forc_lwrad + fv * emg * SB * lw_grnd +
                         4.0 * emg * SB * p3(t_grnd0) * tinc;
    if (io.frac_veg_nosno[p] == 0) io.t_skin[p] = sqrt(sqrt(lw_grnd));
    io.eflx_lwrad_out[p] = lwout;
    io.eflx_lwrad_net[p] = lwout - forc_lwrad;
    io.eflx_sh_grnd[p] = sh;
    io.qflx_evap_soi[p] = ev;
    io.qflx_ev_snow[p] = ev_snow;
    io.qflx_ev_soil[p] = ev_soil;
    io.qflx_ev_h2osfc[p] = ev_h2osfc;
    io.qflx_liqevap_from_top_layer[p] = liqevap;
    io.qflx_solidevap_from_top_layer[p] = solidevap;
    io.qflx_soliddew_to_top_layer[p] = soliddew;
    io.qflx_liqdew_to_top_layer[p] = liqdew;
    io.eflx_soil_grnd[p] = esg;
    io.errsoi_patch[p] = err;
}

// p2c of errsoi over the column's patches (src/main/subgridAveMod.F90:292-320).
__device__ __forceinline__ void soilfluxes_p2c(const ctsmg_soilfluxes_io& io, int c, int begp) {
    const int p0 = io.col_patchi[c] - begp, np = io.col_npatches[c];
    double s = 0.0;
    for (int p = p0; p < p0 + np; ++p) s = s + io.errsoi_patch[p] * io.wtcol[p];
    io.errsoi_col[c] = s;
}
} // namespace ctsmg
