// soil_math.cuh -- constant-base powers shared by the soil-water and heat kernels.
#pragma once
#include <cuda_runtime.h>
#include "fastmath.cuh"

namespace ctsmg {

// Powers with a constant base, as exp of a double-double exponent: the
// product x*ln(base) is formed exactly as hi + lo (FMA error term, Dekker's
// product; ln(base) split into its nearest double and the remainder), and
// exp(hi + lo) is the table-driven exponential with the low part carried into
// its reduced argument.  The result is within about half an ulp of the exact
// power, for one exponential instead of one pow per factor.
constexpr double LN10_HI = 2.302585092994046, LN10_LO = -2.1707562233822494e-16;
constexpr double LN_TKWAT_HI = -0.5621189181535413, LN_TKWAT_LO = 1.1409357209435452e-17;   // ln(0.57)
constexpr double LN_TKICE_HI = 0.8285518175661483, LN_TKICE_LO = 3.2758189660989295e-17;    // ln(2.290)

__device__ __forceinline__ double exp_dd(double hi, double lo) { return fm::exp_dd(hi, lo); }

// 10^x (IceImpedance, SoilWaterMovementMod.F90:2139-2160)
__device__ __forceinline__ double pow10_dd(double x) {
    const double p = x * LN10_HI;
    return exp_dd(p, fma(x, LN10_HI, -p) + x * LN10_LO);
}

// tkwat^a * tkice^b (Johansen saturated conductivity, SoilTemperatureMod.F90:700-705)
__device__ __forceinline__ double tkwat_tkice_pow(double a, double b) {
    const double p1 = a * LN_TKWAT_HI, p2 = b * LN_TKICE_HI;
    const double e1 = fma(a, LN_TKWAT_HI, -p1) + a * LN_TKWAT_LO;
    const double e2 = fma(b, LN_TKICE_HI, -p2) + b * LN_TKICE_LO;
    const double s = p1 + p2, bb = s - p1;                       // TwoSum
    const double es = (p1 - (s - bb)) + (p2 - bb);
    return exp_dd(s, es + e1 + e2);
}

} // namespace ctsmg

