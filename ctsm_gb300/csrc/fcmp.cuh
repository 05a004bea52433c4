// fcmp.cuh -- FP64 comparisons, min and max on the integer pipe.
//
// On GB300 every FP64 warp instruction holds its scheduler's FP64 pipe for
// the same ~64 cycles, whatever it computes, and the column kernels are bound
// by that pipe.  A compare (a branch condition), an fmin / fmax and an
// int-to-double conversion each cost as much as an FMA (measured: a DFMA
// loop with one of them beside every DFMA runs at half the rate, while the
// reciprocal seed rcp.approx.f64 runs on another pipe).  These helpers take
// the same decisions with integer instructions on the operands' bits.  Read
// as sign-magnitude integers and mapped to two's complement (key(-0) =
// key(+0) = 0), the bits of doubles order exactly as their values, so for
// operands that are not NaN
//
//   lt(a, b) == (a < b), le, gt, ge likewise, eq(a, b) == (a == b),
//
// and a NaN operand makes every one of them false, as the IEEE comparison
// does.  min / max follow fmin / fmax (IEEE minNum / maxNum): a NaN operand
// yields the other operand; between equal operands (+0 and -0 included) they
// return the first.  The forms against a literal (ltc, gtc, ... for a
// positive one, ltn, gtn for a negative one, lt0, gt0, ... for zero, minc,
// maxc, max0) need one or two 64-bit integer comparisons and fewer registers
// than the general forms; the GPU tests check every form against the FP64
// instruction over edge cases and random bit patterns, and the CPU tests the
// host build of this header against the host's comparisons.
#pragma once
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define CTSMG_FC_HD __host__ __device__ __forceinline__
#else
#define CTSMG_FC_HD inline
#endif

namespace ctsmg {
namespace ic {

constexpr long long MAG = 0x7fffffffffffffffLL;
constexpr long long INF_BITS = 0x7ff0000000000000LL;

CTSMG_FC_HD long long bits(double x) {
#if defined(__CUDA_ARCH__)
    return __double_as_longlong(x);
#else
    long long b;
    std::memcpy(&b, &x, 8);
    return b;
#endif
}
CTSMG_FC_HD bool isnan_(double x) { return (bits(x) & MAG) > INF_BITS; }
CTSMG_FC_HD long long key(double x) {
    const long long b = bits(x), s = b >> 63;
    return ((b & MAG) ^ s) - s;
}

CTSMG_FC_HD bool lt(double a, double b) { return !isnan_(a) && !isnan_(b) && key(a) < key(b); }
CTSMG_FC_HD bool le(double a, double b) { return !isnan_(a) && !isnan_(b) && key(a) <= key(b); }
CTSMG_FC_HD bool gt(double a, double b) { return lt(b, a); }
CTSMG_FC_HD bool ge(double a, double b) { return le(b, a); }
CTSMG_FC_HD bool eq(double a, double b) { return !isnan_(a) && !isnan_(b) && key(a) == key(b); }
// x != 0.0 (true for NaN, as the IEEE comparison)
CTSMG_FC_HD bool ne0(double x) { return (bits(x) & MAG) != 0; }
// fabs(x) > 0.0 (false for NaN)
CTSMG_FC_HD bool abs_gt0(double x) {
    const long long m = bits(x) & MAG;
    return m != 0 && m <= INF_BITS;
}

// Against a constant: for c > 0 the bits of x, read as a signed integer,
// order like x against c (every negative x, -0 included, reads below), so
// one 64-bit integer comparison decides, with NaN x excluded explicitly.
// The *0 forms compare against +0.0.  c must be a positive literal.
constexpr long long NEG_INF_S = (long long)0xfff0000000000000ULL;   // -inf as a signed integer
CTSMG_FC_HD bool ltc(double x, double c) {
    const long long b = bits(x);
    return b < bits(c) && (b >= 0 || b <= NEG_INF_S);
}
CTSMG_FC_HD bool lec(double x, double c) {
    const long long b = bits(x);
    return b <= bits(c) && (b >= 0 || b <= NEG_INF_S);
}
CTSMG_FC_HD bool gtc(double x, double c) { const long long b = bits(x); return b > bits(c) && b <= INF_BITS; }
CTSMG_FC_HD bool gec(double x, double c) { const long long b = bits(x); return b >= bits(c) && b <= INF_BITS; }
CTSMG_FC_HD bool gt0(double x) { const long long b = bits(x); return b > 0 && b <= INF_BITS; }
CTSMG_FC_HD bool ge0(double x) { const long long b = bits(x); return (b >= 0 && b <= INF_BITS) || b == (long long)0x8000000000000000ULL; }
CTSMG_FC_HD bool lt0(double x) {
    const long long b = bits(x);
    return b < 0 && b != (long long)0x8000000000000000ULL && b <= NEG_INF_S;
}
CTSMG_FC_HD bool le0(double x) { const long long b = bits(x); return b <= 0 && (b == 0 || b <= NEG_INF_S); }
// Against a negative literal c: x < c exactly when x is negative with a
// magnitude above |c| (and not NaN); x > c when x is non-negative (and not
// NaN) or negative with a magnitude below |c|.
CTSMG_FC_HD bool ltn(double x, double c) {
    const long long b = bits(x), m = b & MAG;
    return b < 0 && m > (bits(c) & MAG) && m <= INF_BITS;
}
CTSMG_FC_HD bool gtn(double x, double c) {
    const long long b = bits(x);
    return b >= 0 ? b <= INF_BITS : (b & MAG) < (bits(c) & MAG);
}
// fmax / fmin with a positive constant (a NaN x yields c)
CTSMG_FC_HD double maxc(double x, double c) { return gtc(x, c) ? x : c; }
CTSMG_FC_HD double minc(double x, double c) { return ltc(x, c) ? x : c; }
CTSMG_FC_HD double max0(double x) { return gt0(x) ? x : 0.0; }

// fabs(a) >= fabs(b) (false when either is NaN)
CTSMG_FC_HD bool abs_ge(double a, double b) {
    const long long ma = bits(a) & MAG, mb = bits(b) & MAG;
    return ma <= INF_BITS && mb <= INF_BITS && ma >= mb;
}

CTSMG_FC_HD double min(double a, double b) {
    if (isnan_(a)) return b;
    if (isnan_(b)) return a;
    return key(b) < key(a) ? b : a;
}
CTSMG_FC_HD double max(double a, double b) {
    if (isnan_(a)) return b;
    if (isnan_(b)) return a;
    return key(b) > key(a) ? b : a;
}

} // namespace ic
} // namespace ctsmg
