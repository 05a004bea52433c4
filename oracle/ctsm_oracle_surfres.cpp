// ctsm_oracle_surfres.cpp -- CPU oracle (test infrastructure only) of
// calc_soilevap_resis (src/biogeophys/SurfaceResistanceMod.F90:190-227):
// calc_soil_resistance_sl14 (:330-425) and calc_beta_leepielke1992
// (:231-303) for natural-vegetation soil columns, statement by statement.
// Default-real literals (2.12e-5, 273.15, 1.75, 1.e3) are single precision in
// the reference and are reproduced as (double)(float)x.  Parity unpinned: the
// reference ships no test of these routines.
#include <cmath>
#include <cstdint>
#include <algorithm>
#include "ctsm_gpu.h"
#include "ctsm_oracle.h"
#include "oracle_libm.h"

namespace {
const double DENH2O = 1.000e3, DENICE = 0.917e3;
const double SHR_CONST_PI = 3.14159265358979323846;
const int LS = -CTSMG_NLEVSNO + 1;
using oracle_libm::o_pow;
}

extern "C" int oracle_soilevap_resis(const ctsmg_bounds* b, int num_nolakec, const int32_t* filter_nolakec,
                                     const ctsmg_soilresis_io* io, const ctsmg_soil_resistance_params* par) {
    const int ld = io->ldc;
    for (int fc = 0; fc < num_nolakec; ++fc) {
        const int c = filter_nolakec[fc] - b->begc;
        const size_t s1 = c + (size_t)(1 - LS) * ld, g1 = c;
        const double dz = io->dz[s1], watsat = io->watsat[g1];
        if (par->soil_resis_method == 1) {
            const double vwc_liq = std::max(io->h2osoi_liq[s1], 1.0e-6) / (dz * DENH2O);
            const double eff_por_top = std::max(0.01, watsat - std::min(watsat, io->h2osoi_ice[s1] / (dz * DENICE)));
            const double aird = watsat * o_pow(io->sucsat[g1] / 1.e7, (double)1.f / io->bsw[g1]);
            const double d0 = (double)2.12e-5f * o_pow(io->t_soisno[s1] / (double)273.15f, (double)1.75f);
            const double eps = watsat - aird;
            const double dg = eps * d0 * o_pow(eps / watsat, 3.0 / std::max(3.0, io->bsw[g1]));
            double dsl = par->d_max * std::max(0.001, (par->frac_sat_soil_dsl_init * eff_por_top - vwc_liq)) /
                         std::max(0.001, (par->frac_sat_soil_dsl_init * watsat - aird));
            dsl = std::max(dsl, 0.0);
            dsl = std::min(dsl, 200.0);
            io->dsl[c] = dsl;
            io->soilresis[c] = dsl / (dg * eps * (double)1.e3f) + 20.0;
            io->soilresis[c] = std::min(1.e6, io->soilresis[c]);
        } else {
            const double wx = (io->h2osoi_liq[s1] / DENH2O + io->h2osoi_ice[s1] / DENICE) / dz;
            if (wx < io->watfc[g1]) {
                double fac_fc = std::min(1.0, wx / io->watfc[g1]);
                fac_fc = std::max(fac_fc, 0.01);
                const double q = 1.0 - std::cos(SHR_CONST_PI * fac_fc);
                io->soilbeta[c] = (1.0 - io->frac_sno[c] - io->frac_h2osfc[c]) * 0.25 * (q * q) + io->frac_sno[c] +
                                  io->frac_h2osfc[c];
            } else {
                io->soilbeta[c] = 1.0;
            }
        }
    }
    return 0;
}
