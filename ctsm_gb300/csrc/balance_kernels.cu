// balance_kernels.cu -- per-column water and soil-energy balance errors of a
// model step, as BalanceCheck evaluates them (src/biogeophys/BalanceCheckMod.F90)
// restricted to the scoped calls, with the soil ground heat flux of SoilFluxes
// (src/biogeophys/SoilFluxesMod.F90:170-200, 340-370, 399-430).
#include <cuda_runtime.h>
#include <cstdint>
#include "ctsm_device.cuh"
#include "balance_kernels.cuh"

namespace ctsmg {

__device__ __forceinline__ double ipow4b(double x) { double x2 = x * x; return x2 * x2; }
__device__ __forceinline__ double ipow3b(double x) { double x2 = x * x; return x2 * x; }

__device__ __forceinline__ double column_water(const ctsmg_soiltemp_io& t, int c) {
    const int ld = t.ldc, snl = t.snl[c];
    double w = t.h2osfc[c] + t.h2osno_no_layers[c];
    for (int j = snl + 1; j <= NLEVSOI; ++j) {
        const size_t ix = c + (size_t)(j - LS) * ld;
        w = w + t.h2osoi_liq[ix] + t.h2osoi_ice[ix];
    }
    return w;
}

__global__ void prestep_kernel(ctsmg_soiltemp_io t, int ncol, BalanceState bs) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncol) return;
    const int ld = t.ldc;
    for (int j = t.snl[c] + 1; j <= NLEVGRND; ++j) bs.tssbef[c + (size_t)(j - LS) * ld] = t.t_soisno[c + (size_t)(j - LS) * ld];
    bs.th2osfc_bef[c] = t.t_h2osfc[c];
    bs.w_bef[c] = column_water(t, c);
}

__global__ void balance_kernel(ctsmg_soilwater_io w, ctsmg_soiltemp_io t, int ncol, double dtime, BalanceState bs) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncol) return;
    const int ld = t.ldc, snl = t.snl[c];
    // ---- water: change of column storage minus the scoped fluxes
    // Zeng-Decker: the sink of every soil level, and recharge leaves the
    // column only through the aquifer node (jwt == nlevsoi).  Moisture form:
    // the sink of levels 1..nbedrock, and the bottom flux qcharge unless the
    // boundary is zero-flux.
    const int nl = bs.mf_lbc ? t.nbedrock[c] : NLEVSOI;
    double root = 0.0;
    for (int j = 1; j <= nl; ++j) root = root + w.qflx_rootsoi[c + (size_t)(j - 1) * ld];
    const bool out = bs.mf_lbc ? bs.mf_lbc != 2 : w.zwt[c] > w.zi[c + (size_t)(NLEVSOI + NLEVSNO) * ld];
    const double net = (w.qflx_infl[c] - root - (out ? w.qcharge[c] : 0.0)) * dtime;
    const double errh2o = (column_water(t, c) - bs.w_bef[c]) - net;
    // ---- soil energy: SoilFluxesMod.F90:170-200 (t_grnd0, tinc), 340-370
    // (eflx_soil_grnd) and 399-430 (errsoi), p2c with wtcol
    const double fsno = t.frac_sno_eff[c], fh2o = t.frac_h2osfc[c], emg = t.emg[c], htvp = t.htvp[c];
    const double tb_top = bs.tssbef[c + (size_t)(snl + 1 - LS) * ld], tb_1 = bs.tssbef[c + (size_t)(1 - LS) * ld];
    const double th_bef = bs.th2osfc_bef[c];
    double t_grnd0;
    if (snl < 0) t_grnd0 = fsno * tb_top + (1 - fsno - fh2o) * tb_1 + fh2o * th_bef;
    else t_grnd0 = (1 - fh2o) * tb_1 + fh2o * th_bef;
    const double tinc = t.t_grnd[c] - t_grnd0;
    const double lw_grnd = (fsno * ipow4b(tb_top) + (1.0 - fsno - fh2o) * ipow4b(tb_1) + fh2o * ipow4b(th_bef));
    double store = 0.0;
    for (int j = snl + 1; j <= NLEVGRND; ++j) {
        const size_t ix = c + (size_t)(j - LS) * ld;
        const double d = (t.t_soisno[ix] - bs.tssbef[ix]) / t.fact[ix];
        if (j < 1) store = store - fsno * d;
        else store = store - d;
    }
    const double common = -t.xmf[c] - t.xmf_h2osfc[c] - fh2o * (t.t_h2osfc[c] - th_bef) * (t.c_h2osfc[c] / dtime) +
                          t.eflx_h2osfc_to_snow[c];
    const int p0 = t.col_patchi[c] - 1, np = t.col_npatches[c];
    double errsoi = 0.0;
    for (int p = p0; p < p0 + np; ++p) {
        const double fv = (double)(1 - t.frac_veg_nosno[p]);
        const double sh = t.eflx_sh_grnd[p], ev = t.qflx_evap_soi[p];
        const double eflx_soil_grnd = ((1.0 - fsno) * t.sabg_soil[p] + fsno * t.sabg_snow[p]) + t.dlrad[p] +
                                      fv * emg * t.forc_lwrad[c] - emg * SB * lw_grnd -
                                      emg * SB * ipow3b(t_grnd0) * (4.0 * tinc) - (sh + ev * htvp) - tinc * t.cgrnd[p];
        errsoi = errsoi + (eflx_soil_grnd + common + store) * t.wtcol[p];
    }
    bs.errh2o[c] = errh2o;
    bs.errsoi[c] = errsoi;
    if (*bs.step >= bs.skip_steps) {
        bs.errh2o_max[c] = fmax(bs.errh2o_max[c], fabs(errh2o));
        bs.errsoi_max[c] = fmax(bs.errsoi_max[c], fabs(errsoi));
    }
}

__global__ void step_count_kernel(int* step) { *step = *step + 1; }

cudaError_t launch_prestep(const ctsmg_soiltemp_io& t, int ncol, const BalanceState& bs, cudaStream_t s) {
    prestep_kernel<<<(ncol + 127) / 128, 128, 0, s>>>(t, ncol, bs);
    return cudaGetLastError();
}

cudaError_t launch_balance(const ctsmg_soilwater_io& w, const ctsmg_soiltemp_io& t, int ncol, double dtime,
                           const BalanceState& bs, cudaStream_t s) {
    balance_kernel<<<(ncol + 127) / 128, 128, 0, s>>>(w, t, ncol, dtime, bs);
    step_count_kernel<<<1, 1, 0, s>>>(bs.step);
    return cudaGetLastError();
}

} // namespace ctsmg
