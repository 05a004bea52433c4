// surface_resistance.cuh -- calc_soilevap_resis for one soil column
// (src/biogeophys/SurfaceResistanceMod.F90:190-227): the sl_14 dry surface
// layer resistance (:330-425) or the leepielke_1992 evaporation factor
// (:231-303).  Shared by the drop-in kernel and the resident step.
#pragma once
#include <cuda_runtime.h>
#include "ctsm_gpu.h"
#include "ctsm_device.cuh"
#include "fastmath.cuh"

namespace ctsmg {

struct SoilResisArgs {
    int method;                      // 1 sl_14, 0 leepielke_1992
    double d_max, frac_sat_soil_dsl_init;
    const double* d_max_c = nullptr; // per-column d_max (resident ensembles) or NULL
};

// Default-real literals of the reference (2.12e-5, 273.15) as the single
// precision values the Fortran compiler stores.
__device__ __forceinline__ void soilevap_resis_column(const ctsmg_soilresis_io& io, int c, const SoilResisArgs& a) {
    const int ld = io.ldc;
    const size_t s1 = c + (size_t)(1 - LS) * ld, g1 = c;
    const double dz = io.dz[s1], ws = io.watsat[g1];
    if (a.method == 1) {
        const double vwc_liq = fmax(io.h2osoi_liq[s1], 1.0e-6) / (dz * DENH2O);
        const double vi = io.h2osoi_ice[s1] / (dz * DENICE);
        const double eff_por_top = fmax(0.01, ws - ((vi < ws) ? vi : ws));
        const double bsw = io.bsw[g1];
        const double aird = ws * fm::pow(io.sucsat[g1] / 1.e7, 1.0 / bsw);
        const double d0 = (double)2.12e-5f * fm::pow(io.t_soisno[s1] / (double)273.15f, 1.75);
        const double eps = ws - aird;
        const double dg = eps * d0 * fm::pow(eps / ws, 3.0 / fmax(3.0, bsw));
        double dsl = (a.d_max_c ? a.d_max_c[c] : a.d_max) * fmax(0.001, (a.frac_sat_soil_dsl_init * eff_por_top - vwc_liq)) /
                     fmax(0.001, (a.frac_sat_soil_dsl_init * ws - aird));
        dsl = fmax(dsl, 0.0);
        dsl = fmin(dsl, 200.0);
        io.dsl[c] = dsl;
        const double r = dsl / (dg * eps * 1.e3) + 20.0;
        io.soilresis[c] = fmin(1.e6, r);
    } else {
        const double wx = (io.h2osoi_liq[s1] / DENH2O + io.h2osoi_ice[s1] / DENICE) / dz;
        const double wfc = io.watfc[g1];
        if (wx < wfc) {
            double fac_fc = fmin(1.0, wx / wfc);
            fac_fc = fmax(fac_fc, 0.01);
            const double fs = io.frac_sno[c], fh = io.frac_h2osfc[c];
            const double q = 1.0 - cos(CTSMG_PI * fac_fc);
            io.soilbeta[c] = (1.0 - fs - fh) * 0.25 * (q * q) + fs + fh;
        } else {
            io.soilbeta[c] = 1.0;
        }
    }
}

cudaError_t launch_soilevap_resis(const ctsmg_soilresis_io& io, int begc, int nfilt, const int32_t* d_filt,
                                  const SoilResisArgs& a, cudaStream_t s);

} // namespace ctsmg
