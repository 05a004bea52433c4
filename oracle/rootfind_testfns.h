// rootfind_testfns.h -- synthetic functions for checking the Ci root finder
// (PhotosynthesisMod.F90:2251-2485) outside Photosynthesis.  Test support:
// included by the oracle and by the root-finder test harness so that both
// evaluate bit-identical functions.  prm holds up to four coefficients.
#pragma once
#include <cmath>

static inline double rf_testfn(int k, const double* prm, double x) {
    switch (k) {
    case 0: return x - prm[0];                                          // secant lands on the root
    case 1: return 1.e-3 * (x - prm[0]) + 0.5 * std::tanh((x - prm[0]) / prm[1]);
    case 2: return (x - prm[0]) * (x - prm[0]) / prm[1] + prm[2];       // no root: iteration limit
    case 3: return std::fmax(0.0, x - prm[0]);                          // exact zeros
    case 4: return std::atan((x - prm[0]) / prm[1]);                    // overshoot, Brent
    default: return prm[0] * (x - prm[1]) + prm[2] * std::sin(x / prm[3]);
    }
}
