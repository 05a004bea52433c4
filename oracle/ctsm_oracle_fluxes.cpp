// ctsm_oracle_fluxes.cpp -- CPU oracle (test infrastructure only) for
// SoilFluxes, src/biogeophys/SoilFluxesMod.F90:163-518, natural-vegetation
// patches, and the filtered p2c of src/main/subgridAveMod.F90:292-320.
// Statements and evaluation order follow the reference loops; Fortran's x**3
// and x**4 are x*x*x and (x*x)*(x*x), a*b/c is (a*b)/c.
#include <cmath>
#include <cstdint>
#include <vector>
#include "ctsm_gpu.h"
#include "ctsm_oracle.h"

namespace {
const double TFRZ = 273.15, SB = 5.67e-8, HVAP = 2.501e6;
const int NLEVSNO = 12, NLEVGRND = 25, LS = -NLEVSNO + 1;
double p3(double x) { return x * x * x; }
double p4(double x) { const double x2 = x * x; return x2 * x2; }
}

extern "C" int oracle_soilfluxes(const ctsmg_bounds* b, int num_nolakec, const int32_t* filter_nolakec,
                                 int num_nolakep, const int32_t* filter_nolakep, const ctsmg_soilfluxes_io* io,
                                 double dtime) {
    const int ld = io->ldc;
    auto SS = [&](const double* a, int c, int j) { return a[c + (size_t)(j - LS) * ld]; };
    const int ncol = b->endc - b->begc + 1;
    std::vector<double> tinc(ncol), t_grnd0(ncol);
    // :168-185
    for (int fc = 0; fc < num_nolakec; ++fc) {
        const int c = filter_nolakec[fc] - b->begc;
        const int snl = io->snl[c];
        const double fs = io->frac_sno_eff[c], fh = io->frac_h2osfc[c];
        if (snl < 0)
            t_grnd0[c] = fs * SS(io->tssbef, c, snl + 1) + (1 - fs - fh) * SS(io->tssbef, c, 1) + fh * io->t_h2osfc_bef[c];
        else
            t_grnd0[c] = (1 - fh) * SS(io->tssbef, c, 1) + fh * io->t_h2osfc_bef[c];
        tinc[c] = io->t_grnd[c] - t_grnd0[c];
    }
    // :189-205
    for (int fp = 0; fp < num_nolakep; ++fp) {
        const int p = filter_nolakep[fp] - b->begp, c = io->patch_column[p] - b->begc;
        io->eflx_sh_grnd[p] = io->eflx_sh_grnd[p] + tinc[c] * io->cgrnds[p];
        io->qflx_evap_soi[p] = io->qflx_evap_soi[p] + tinc[c] * io->cgrndl[p];
        io->qflx_ev_snow[p] = io->qflx_ev_snow[p] + tinc[c] * io->cgrndl[p];
        io->qflx_ev_soil[p] = io->qflx_ev_soil[p] + tinc[c] * io->cgrndl[p];
        io->qflx_ev_h2osfc[p] = io->qflx_ev_h2osfc[p] + tinc[c] * io->cgrndl[p];
    }
    // :209-274
    for (int fp = 0; fp < num_nolakep; ++fp) {
        const int p = filter_nolakep[fp] - b->begp, c = io->patch_column[p] - b->begc;
        const int j = io->snl[c] + 1;
        io->qflx_liqevap_from_top_layer[p] = 0.0;
        io->qflx_solidevap_from_top_layer[p] = 0.0;
        io->qflx_soliddew_to_top_layer[p] = 0.0;
        io->qflx_liqdew_to_top_layer[p] = 0.0;
        const double liq = SS(io->h2osoi_liq, c, j), ice = SS(io->h2osoi_ice, c, j);
        if (io->qflx_ev_snow[p] >= 0.0) {
            if ((liq + ice) > 0.0)
                io->qflx_liqevap_from_top_layer[p] = std::fmax(io->qflx_ev_snow[p] * (liq / (liq + ice)), 0.0);
            else
                io->qflx_liqevap_from_top_layer[p] = 0.0;
            io->qflx_solidevap_from_top_layer[p] = io->qflx_ev_snow[p] - io->qflx_liqevap_from_top_layer[p];
        } else {
            if (io->t_grnd[c] < TFRZ) io->qflx_soliddew_to_top_layer[p] = std::fabs(io->qflx_ev_snow[p]);
            else io->qflx_liqdew_to_top_layer[p] = std::fabs(io->qflx_ev_snow[p]);
        }
    }
    // :277-329
    for (int fp = 0; fp < num_nolakep; ++fp) {
        const int p = filter_nolakep[fp] - b->begp, c = io->patch_column[p] - b->begc;
        const int j = io->snl[c] + 1;
        const double liq = SS(io->h2osoi_liq, c, j), ice = SS(io->h2osoi_ice, c, j);
        const double fs = io->frac_sno_eff[c], fh = io->frac_h2osfc[c];
        if (j < 1) {
            const double lim = (ice + liq) / (fs * dtime);
            if (io->qflx_ev_snow[p] > lim) {
                const double demand = io->qflx_ev_snow[p];
                io->qflx_ev_snow[p] = lim;
                io->qflx_evap_soi[p] = io->qflx_evap_soi[p] - fs * (demand - lim);
                io->qflx_liqevap_from_top_layer[p] = std::fmax(liq / (fs * dtime), 0.0);
                io->qflx_solidevap_from_top_layer[p] = std::fmax(ice / (fs * dtime), 0.0);
                io->eflx_sh_grnd[p] = io->eflx_sh_grnd[p] + fs * (demand - lim) * io->htvp[c];
            }
        }
        if (j == 1 && fh < 1.0) {
            const double lim = ice / (dtime * (1.0 - fh));
            if (io->qflx_solidevap_from_top_layer[p] >= lim) {
                const double demand = io->qflx_solidevap_from_top_layer[p];
                io->qflx_solidevap_from_top_layer[p] = lim;
                io->qflx_liqevap_from_top_layer[p] = io->qflx_liqevap_from_top_layer[p] + (demand - lim);
            }
        }
    }
    // :334-395
    for (int fp = 0; fp < num_nolakep; ++fp) {
        const int p = filter_nolakep[fp] - b->begp, c = io->patch_column[p] - b->begc;
        const int snl = io->snl[c];
        const double fs = io->frac_sno_eff[c], fh = io->frac_h2osfc[c], emg = io->emg[c];
        const double lw_grnd = (fs * p4(SS(io->tssbef, c, snl + 1)) + (1.0 - fs - fh) * p4(SS(io->tssbef, c, 1)) +
                                fh * p4(io->t_h2osfc_bef[c]));
        io->eflx_soil_grnd[p] = ((1.0 - fs) * io->sabg_soil[p] + fs * io->sabg_snow[p]) + io->dlrad[p] +
                                (1 - io->frac_veg_nosno[p]) * emg * io->forc_lwrad[c] - emg * SB * lw_grnd -
                                emg * SB * p3(t_grnd0[c]) * (4.0 * tinc[c]) -
                                (io->eflx_sh_grnd[p] + io->qflx_evap_soi[p] * io->htvp[c]);
        io->eflx_sh_tot[p] = io->eflx_sh_veg[p] + io->eflx_sh_grnd[p];
        io->qflx_evap_tot[p] = io->qflx_evap_veg[p] + io->qflx_evap_soi[p];
        io->eflx_lh_tot[p] = HVAP * io->qflx_evap_veg[p] + io->htvp[c] * io->qflx_evap_soi[p];
        io->qflx_evap_can[p] = io->qflx_evap_veg[p] - io->qflx_tran_veg[p];
        io->eflx_lh_vege[p] = (io->qflx_evap_veg[p] - io->qflx_tran_veg[p]) * HVAP;
        io->eflx_lh_vegt[p] = io->qflx_tran_veg[p] * HVAP;
        io->eflx_lh_grnd[p] = io->qflx_evap_soi[p] * io->htvp[c];
    }
    // :401-429
    for (int fp = 0; fp < num_nolakep; ++fp) {
        const int p = filter_nolakep[fp] - b->begp, c = io->patch_column[p] - b->begc;
        const double fh = io->frac_h2osfc[c];
        io->errsoi_patch[p] = io->eflx_soil_grnd[p] - io->xmf[c] - io->xmf_h2osfc[c] -
                              fh * (io->t_h2osfc[c] - io->t_h2osfc_bef[c]) * (io->c_h2osfc[c] / dtime);
        io->errsoi_patch[p] = io->errsoi_patch[p] + io->eflx_h2osfc_to_snow[c];
    }
    for (int j = -NLEVSNO + 1; j <= NLEVGRND; ++j) {
        for (int fp = 0; fp < num_nolakep; ++fp) {
            const int p = filter_nolakep[fp] - b->begp, c = io->patch_column[p] - b->begc;
            const int snl = io->snl[c];
            const double d = SS(io->t_soisno, c, j) - SS(io->tssbef, c, j);
            if (j >= snl + 1 && j < 1) io->errsoi_patch[p] = io->errsoi_patch[p] - io->frac_sno_eff[c] * d / SS(io->fact, c, j);
            if (j >= 1) io->errsoi_patch[p] = io->errsoi_patch[p] - d / SS(io->fact, c, j);
        }
    }
    // :457-496
    for (int fp = 0; fp < num_nolakep; ++fp) {
        const int p = filter_nolakep[fp] - b->begp, c = io->patch_column[p] - b->begc;
        const int snl = io->snl[c];
        const double fs = io->frac_sno_eff[c], fh = io->frac_h2osfc[c], emg = io->emg[c];
        const double lw_grnd = (fs * p4(SS(io->tssbef, c, snl + 1)) + (1.0 - fs - fh) * p4(SS(io->tssbef, c, 1)) +
                                fh * p4(io->t_h2osfc_bef[c]));
        const int fv = 1 - io->frac_veg_nosno[p];
        io->eflx_lwrad_out[p] = io->ulrad[p] + fv * (1. - emg) * io->forc_lwrad[c] + fv * emg * SB * lw_grnd +
                                4.0 * emg * SB * p3(t_grnd0[c]) * tinc[c];
        if (io->frac_veg_nosno[p] == 0) io->t_skin[p] = std::sqrt(std::sqrt(lw_grnd));
        io->eflx_lwrad_net[p] = io->eflx_lwrad_out[p] - io->forc_lwrad[c];
    }
    // p2c (subgridAveMod.F90:292-320)
    for (int fc = 0; fc < num_nolakec; ++fc) {
        const int c = filter_nolakec[fc] - b->begc;
        io->errsoi_col[c] = 0.0;
        for (int p = io->col_patchi[c] - b->begp; p < io->col_patchi[c] - b->begp + io->col_npatches[c]; ++p)
            io->errsoi_col[c] = io->errsoi_col[c] + io->errsoi_patch[p] * io->wtcol[p];
    }
    return 0;
}
