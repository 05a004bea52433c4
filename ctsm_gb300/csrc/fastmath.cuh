// fastmath.cuh -- table-driven FP64 log, exp and pow for the column kernels.
//
// GB300 issues FP64 at a small fraction of its FP32/integer rate, and the
// soil and canopy kernels spend most of their FP64 instructions in pow, log
// and exp (the Clapp-Hornberger retention curve alone is two powers per
// level and Newton pass).  These forms move everything but the core
// arithmetic to integer instructions and table loads:
//
//   log  -- Tang, "Table-driven implementation of the logarithm function in
//           IEEE floating-point arithmetic", ACM TOMS 16(4), 1990:
//           x = 2^k m, m in [1,2); F = 1 + j/256 nearest to m; f = m - F
//           (exact); r = f / F (via a tabulated 1/F), |r| <= 2^-9;
//           ln x = k ln2 + ln F + log1p(r), log1p by its Taylor series to
//           r^6 (truncation < 2^-66).  k ln2 + ln F is exact (both on a
//           2^-42 grid), and the result is returned as an unevaluated sum
//           hi + lo so that pow keeps ~60 bits of the logarithm.
//   exp  -- Tang, "Table-driven implementation of the exponential function
//           in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989:
//           t = (128 m + j) ln2/128 + r, |r| <= ln2/256; exp(t) =
//           2^m 2^(j/128) (1 + expm1(r)), expm1 by its Taylor series to r^5
//           (truncation < 2^-63), the scale by 2^m on the exponent bits.
//   pow  -- exp(y ln x) with the double-double logarithm and the product's
//           FMA error term carried into the exponential's reduced argument.
//
// Every floating-point operation is written as an explicitly rounded
// intrinsic, so the device result is bit-identical to the host build of this
// header (compiled without contraction); the tests compare the two and bound
// the error against 80-digit references.  Arguments outside the fast range
// (zero, negative, subnormal, infinite or NaN x; |y ln x| >= 704) take the
// CUDA math library's function, so special cases follow C99.
#pragma once
#include <cmath>
#include <cstring>
#include <cstdint>
#include "fastmath_tables.h"

#if defined(__CUDACC__)
#define CTSMG_FM_HD __host__ __device__ __forceinline__
#else
#define CTSMG_FM_HD inline
#endif

namespace ctsmg {
namespace fm {

#if defined(__CUDACC__)
static __device__ const double LOG_INVF_D[] = CTSMG_FM_LOG_INVF;
static __device__ const double2 LOG_HILO_D[] = CTSMG_FM_LOG_HILO;
static __device__ const double2 EXP_HILO_D[] = CTSMG_FM_EXP_HILO;
#endif
struct HiLo { double hi, lo; };
static const double LOG_INVF_H[] = CTSMG_FM_LOG_INVF;
static const HiLo LOG_HILO_H[] = CTSMG_FM_LOG_HILO;
static const HiLo EXP_HILO_H[] = CTSMG_FM_EXP_HILO;

CTSMG_FM_HD int64_t bits(double x) {
#if defined(__CUDA_ARCH__)
    return __double_as_longlong(x);
#else
    int64_t i; std::memcpy(&i, &x, 8); return i;
#endif
}
CTSMG_FM_HD double from_bits(int64_t i) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double(i);
#else
    double x; std::memcpy(&x, &i, 8); return x;
#endif
}
#if defined(__CUDA_ARCH__)
CTSMG_FM_HD double add(double a, double b) { return __dadd_rn(a, b); }
CTSMG_FM_HD double sub(double a, double b) { return __dsub_rn(a, b); }
CTSMG_FM_HD double mul(double a, double b) { return __dmul_rn(a, b); }
CTSMG_FM_HD double fma_(double a, double b, double c) { return __fma_rn(a, b, c); }
// (double)k for any int, built on the integer pipe (an int-to-FP64
// conversion is an FP64-pipe instruction): exact, as the conversion
CTSMG_FM_HD double i2d(int k) {
    const unsigned a = k < 0 ? 0u - (unsigned)k : (unsigned)k;
    const int e = 31 - __clz(a | 1u);                            // a in [2^e, 2^(e+1)) for a > 0
    const uint64_t m = ((uint64_t)a << (52 - e)) & 0x000FFFFFFFFFFFFFULL;
    const uint64_t b = ((uint64_t)(k < 0) << 63) | ((uint64_t)(1023 + e) << 52) | m;
    return k == 0 ? 0.0 : __longlong_as_double((long long)b);
}
CTSMG_FM_HD double invf(int j) { return __ldg(&LOG_INVF_D[j]); }
CTSMG_FM_HD HiLo loghl(int j) { const double2 t = __ldg(&LOG_HILO_D[j]); return {t.x, t.y}; }
CTSMG_FM_HD HiLo exphl(int j) { const double2 t = __ldg(&EXP_HILO_D[j]); return {t.x, t.y}; }
CTSMG_FM_HD double lib_log(double x) { return ::log(x); }
CTSMG_FM_HD double lib_exp(double x) { return ::exp(x); }
CTSMG_FM_HD double lib_pow(double x, double y) { return ::pow(x, y); }
CTSMG_FM_HD double lib_log10(double x) { return ::log10(x); }
#else
inline double add(double a, double b) { return a + b; }
inline double sub(double a, double b) { return a - b; }
inline double mul(double a, double b) { return a * b; }
inline double fma_(double a, double b, double c) { return std::fma(a, b, c); }
inline double i2d(int k) { return (double)k; }
inline double invf(int j) { return LOG_INVF_H[j]; }
inline HiLo loghl(int j) { return LOG_HILO_H[j]; }
inline HiLo exphl(int j) { return EXP_HILO_H[j]; }
inline double lib_log(double x) { return std::log(x); }
inline double lib_exp(double x) { return std::exp(x); }
inline double lib_pow(double x, double y) { return std::pow(x, y); }
inline double lib_log10(double x) { return std::log10(x); }
#endif

constexpr double LN2_HI = CTSMG_FM_LN2_HI, LN2_LO = CTSMG_FM_LN2_LO;
constexpr double EXP_INVL = CTSMG_FM_EXP_INVL, EXP_L1 = CTSMG_FM_EXP_L1, EXP_L2 = CTSMG_FM_EXP_L2;
constexpr double INV_LN10_HI = CTSMG_FM_INV_LN10_HI, INV_LN10_LO = CTSMG_FM_INV_LN10_LO;
constexpr double SHIFT = 0x1.8p52;      // z = t*128/ln2 + SHIFT rounds to an integer in the low bits
constexpr int64_t EXP_ONE = 0x3FF0000000000000LL;
constexpr int LOG_SH = 52 - CTSMG_FM_LOG_BITS;
constexpr int EXP_N = 1 << CTSMG_FM_EXP_BITS;

// x is positive, normal and finite
CTSMG_FM_HD bool log_fast(int64_t hx) {
    return (uint64_t)(hx - 0x0010000000000000LL) < 0x7FE0000000000000ULL;
}
// |t| < 704: 2^m stays normal for both the result and its reciprocal
CTSMG_FM_HD bool exp_fast(double t) {
    return ((uint32_t)((uint64_t)bits(t) >> 32) & 0x7fffffffu) < 0x40860000u;
}

// ln x = hi + lo for a positive normal finite x (log_fast), |lo| <= ulp(hi)
CTSMG_FM_HD double log_dd_fast(int64_t hx, double& lo) {
    const int k = (int)(hx >> 52) - 1023;
    const int64_t mant = hx & 0x000FFFFFFFFFFFFFLL;
    const int j = (int)((mant + (1LL << (LOG_SH - 1))) >> LOG_SH);
    const double m = from_bits(mant | EXP_ONE);
    const double F = from_bits(EXP_ONE + ((int64_t)j << LOG_SH));
    const double f = sub(m, F);                                   // exact (Sterbenz)
    const double r = mul(f, invf(j));
    const double kd = i2d(k);
    const HiLo t = loghl(j);
    const double A = fma_(kd, LN2_HI, t.hi);                      // exact on the 2^-42 grid
    const double B = fma_(kd, LN2_LO, t.lo);
    const double r2 = mul(r, r);
    double p = fma_(r, -1.0 / 6.0, 0.2);
    p = fma_(r, p, -0.25);
    p = fma_(r, p, 1.0 / 3.0);
    p = fma_(r, p, -0.5);                                         // log1p(r) = r + r^2 p
    const double q = fma_(r2, p, B);
    const double hi = add(A, r);                                  // |A| >= |r| or A == 0: Fast2Sum
    lo = add(add(sub(A, hi), r), q);
    return hi;
}

// exp(h + l), |h| < 704 (exp_fast), |l| <= 2^-40 |h| or so
CTSMG_FM_HD double exp_dd_fast(double h, double l) {
    const double z = fma_(h, EXP_INVL, SHIFT);
    const int n = (int)(uint32_t)(uint64_t)bits(z);
    const double nd = sub(z, SHIFT);
    double r = fma_(nd, -EXP_L1, h);
    r = add(fma_(nd, -EXP_L2, r), l);
    const double r2 = mul(r, r);
    double p = fma_(r, 1.0 / 120.0, 1.0 / 24.0);
    p = fma_(r, p, 1.0 / 6.0);
    p = fma_(r, p, 0.5);
    p = fma_(r2, p, r);                                           // expm1(r)
    const HiLo t = exphl(n & (EXP_N - 1));
    const double R = add(t.hi, fma_(t.hi, p, t.lo));
    return from_bits(bits(R) + ((int64_t)(n >> CTSMG_FM_EXP_BITS) << 52));
}

CTSMG_FM_HD double log(double x) {
    const int64_t hx = bits(x);
    if (!log_fast(hx)) return lib_log(x);
    double lo;
    const double hi = log_dd_fast(hx, lo);
    return add(hi, lo);
}

CTSMG_FM_HD double log10(double x) {
    const int64_t hx = bits(x);
    if (!log_fast(hx)) return lib_log10(x);
    double lo;
    const double hi = log_dd_fast(hx, lo);
    return fma_(hi, INV_LN10_HI, fma_(hi, INV_LN10_LO, mul(lo, INV_LN10_HI)));
}

CTSMG_FM_HD double exp(double x) {
    if (!exp_fast(x)) return lib_exp(x);
    return exp_dd_fast(x, 0.0);
}

// exp(hi + lo) for an unevaluated double-double exponent
CTSMG_FM_HD double exp_dd(double hi, double lo) {
    if (!exp_fast(hi)) { const double e = lib_exp(hi); return fma_(e, lo, e); }
    return exp_dd_fast(hi, lo);
}

CTSMG_FM_HD double pow(double x, double y) {
    const int64_t hx = bits(x);
    if (!log_fast(hx)) return lib_pow(x, y);
    double lo;
    const double hi = log_dd_fast(hx, lo);
    const double ph = mul(y, hi);
    if (!exp_fast(ph)) return lib_pow(x, y);
    const double pl = fma_(y, lo, fma_(y, hi, -ph));
    return exp_dd_fast(ph, pl);
}

} // namespace fm
} // namespace ctsmg
