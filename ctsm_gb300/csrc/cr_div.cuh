// cr_div.cuh -- correctly rounded FP64 quotients that share one reciprocal.
//
// The soil kernels divide many numerators by the same denominator (the layer
// spacing z(j+1)-z(j) in the heat flux, the matrix rows and the post-solve
// flux; dtime; the porosity; the pivot of each elimination step), and every
// FP64 instruction counts on GB300: an IEEE division is 8 FP64-pipe
// instructions (measured).  Here a quotient is formed from an approximate
// reciprocal y of b, computed once per divisor, and one Newton-Markstein
// correction (P. Markstein, "Computation of elementary functions on the IBM
// RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990; J.-M. Muller et
// al., Handbook of Floating-Point Arithmetic, 2nd ed., 2018, sec. 4.7):
//
//   q0 = RN(a y),  r = RN(a - b q0) (one FMA),  q = RN(q0 + r y) (one FMA).
//
// On the device y is the special-function unit's reciprocal seed
// (rcp.approx.ftz.f64, relative error below 2^-19.9, measured) refined by one
// Newton step y1 = y0 + y0 (1 - b y0): relative error e1 below 2^-39.8.  Then
// q0 = (a/b)(1 + e1)(1 + e2), |e2| <= 2^-53, and the exact value before the
// last rounding is (a/b)(1 - h (e1 + e3 + e1 e3)) with h = e1 + e2 + e1 e2 and
// |e3| <= 2^-53: within 2^-79 |a/b| of a/b, so q is RN(a/b) -- the same bits
// as the division -- unless a/b lies within 2^-79 |a/b| of the midpoint
// between two doubles, where it may be the other neighbour (one ulp).  A
// reciprocal costs 2 FP64 instructions and a quotient 3 (a division 8).  The
// host build (the tests' reference for this header) uses y = RN(1/b).  Zero,
// subnormal, huge, infinite and NaN operands (biased exponent of a or b
// outside [0x201, 0x5fe], checked with integer instructions) take the
// ordinary division, so special values behave exactly as a / b.
#pragma once
#include <cstring>

#if defined(__CUDACC__)
#define CTSMG_CRD_HD __host__ __device__ __forceinline__
#else
#define CTSMG_CRD_HD inline
#endif

namespace ctsmg {

struct Recip {
    double b, y;   // divisor and its reciprocal (RN(1/b) on the host, within 2^-39.8 on the device)
    int ok;        // b inside the exponent range of the fast path
};

CTSMG_CRD_HD int crdiv_in_range(double x) {
#ifdef __CUDA_ARCH__
    const unsigned e = ((unsigned)__double2hiint(x) >> 20) & 0x7ffu;
#else
    unsigned long long u;
    std::memcpy(&u, &x, 8);
    const unsigned e = (unsigned)(u >> 52) & 0x7ffu;
#endif
    return (e - 0x201u) <= (0x5feu - 0x201u);
}

CTSMG_CRD_HD Recip recip(double b) {
    Recip r;
    r.b = b;
#ifdef __CUDA_ARCH__
    double y0;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y0) : "d"(b));
    r.y = __fma_rn(y0, __fma_rn(-b, y0, 1.0), y0);
#else
    r.y = 1.0 / b;
#endif
    r.ok = crdiv_in_range(b);
    return r;
}

// a / R.b: RN(a/b) except within 2^-79 |a/b| of a rounding midpoint.
CTSMG_CRD_HD double divr(double a, const Recip& R) {
    if (!(R.ok & crdiv_in_range(a))) return a / R.b;
#ifdef __CUDA_ARCH__
    const double q = __dmul_rn(a, R.y);
    return __fma_rn(__fma_rn(-R.b, q, a), R.y, q);
#else
    const double q = a * R.y;
    return __builtin_fma(__builtin_fma(-R.b, q, a), R.y, q);
#endif
}

// 0.0 / b: the signed zero for b of normal, in-range magnitude (integer
// instructions only), else the division itself (0/0, 0/inf, 0/NaN, ...).
CTSMG_CRD_HD double zero_over(double b) {
#ifdef __CUDA_ARCH__
    return crdiv_in_range(b) ? __hiloint2double(__double2hiint(b) & (int)0x80000000, 0) : 0.0 / b;
#else
    if (!crdiv_in_range(b)) return 0.0 / b;
    return (b < 0.0) ? -0.0 : 0.0;
#endif
}

// a / b through a reciprocal of its own: 5 FP64 instructions against 8.
CTSMG_CRD_HD double divf(double a, double b) { return divr(a, recip(b)); }

// A constant divisor with its reciprocal RN(1/b) formed by the compiler.
#define CTSMG_CONST_RECIP(b) (::ctsmg::Recip{(b), 1.0 / (b), 1})

} // namespace ctsmg
