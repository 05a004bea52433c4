// cr_div.cuh -- correctly rounded FP64 quotients that share one reciprocal.
//
// The soil kernels divide many numerators by the same denominator (the layer
// spacing z(j+1)-z(j) in the heat flux, the matrix rows and the post-solve
// flux; dtime; the porosity; the band-LU pivot in the back substitution).  On
// GB300 an FP64 division is 8 FP64-pipe instructions and the correctly rounded
// reciprocal RN(1/b) 5 (measured), so a quotient is formed here from y =
// RN(1/b), computed once per divisor, by one Newton-Markstein correction
// (P. Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Dev. 34(1), 1990; J.-M. Muller et al.,
// Handbook of Floating-Point Arithmetic, 2nd ed., 2018, sec. 4.7):
//
//   q0 = RN(a y),  r = RN(a - b q0) (one FMA),  q = RN(q0 + r y) (one FMA).
//
// With y = (1/b)(1 + e1), q0 = (a/b)(1 + e1)(1 + e2) and r = RN(a - b q0),
// |e_i| <= u = 2^-53, the exact value before the last rounding is
// (a/b)(1 + d) with |d| <= (2u + u^2)^2 (1 + u) < 2^-103.9, so q is RN(a/b)
// -- the same bits as the division -- unless a/b lies within 2^-103.9 |a/b|
// of the midpoint between two doubles, where it may be the other neighbour
// (one ulp).  Three FP64 instructions per quotient.  Zero, subnormal, huge,
// infinite and NaN operands (biased exponent of a or b outside [0x201,
// 0x5fe], checked with integer instructions) take the ordinary division, so
// special values behave exactly as a / b.
#pragma once
#include <cstring>

#if defined(__CUDACC__)
#define CTSMG_CRD_HD __host__ __device__ __forceinline__
#else
#define CTSMG_CRD_HD inline
#endif

namespace ctsmg {

struct Recip {
    double b, y;   // divisor and RN(1/b)
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
    r.y = __drcp_rn(b);
#else
    r.y = 1.0 / b;
#endif
    r.ok = crdiv_in_range(b);
    return r;
}

// a / R.b: RN(a/b) except within 2^-103.9 |a/b| of a rounding midpoint.
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

// A constant divisor with its reciprocal RN(1/b) formed by the compiler.
#define CTSMG_CONST_RECIP(b) (::ctsmg::Recip{(b), 1.0 / (b), 1})

} // namespace ctsmg
