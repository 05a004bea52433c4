// fcmp.cuh -- FP64 comparisons, min and max on the integer pipe.
//
// On GB300 every FP64 warp instruction holds its scheduler's FP64 pipe for
// the same ~64 cycles, whatever it computes, and the column kernels are bound
// by that pipe: an FP64 compare (a branch condition) or an fmin / fmax costs
// as much as an FMA.  These helpers take the same decisions with integer
// instructions on the operands' bits.  Read as sign-magnitude integers and
// mapped to two's complement (key(-0) = key(+0) = 0), the bits of doubles
// order exactly as their values, so for operands that are not NaN
//
//   lt(a, b) == (a < b), le, gt, ge likewise, eq(a, b) == (a == b),
//
// and a NaN operand makes every one of them false, as the IEEE comparison
// does.  min / max follow fmin / fmax (IEEE minNum / maxNum): a NaN operand
// yields the other operand; between equal operands (+0 and -0 included) they
// return the first.  Comparisons against a literal fold its key at compile
// time, so they cost a few integer instructions and no FP64 instruction.
#pragma once
#include <cstdint>

namespace ctsmg {
namespace ic {

constexpr long long MAG = 0x7fffffffffffffffLL;
constexpr long long INF_BITS = 0x7ff0000000000000LL;

__device__ __forceinline__ long long bits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ bool isnan_(double x) { return (bits(x) & MAG) > INF_BITS; }
__device__ __forceinline__ long long key(double x) {
    const long long b = bits(x), s = b >> 63;
    return ((b & MAG) ^ s) - s;
}

__device__ __forceinline__ bool lt(double a, double b) { return !isnan_(a) && !isnan_(b) && key(a) < key(b); }
__device__ __forceinline__ bool le(double a, double b) { return !isnan_(a) && !isnan_(b) && key(a) <= key(b); }
__device__ __forceinline__ bool gt(double a, double b) { return lt(b, a); }
__device__ __forceinline__ bool ge(double a, double b) { return le(b, a); }
__device__ __forceinline__ bool eq(double a, double b) { return !isnan_(a) && !isnan_(b) && key(a) == key(b); }
// x != 0.0 (true for NaN, as the IEEE comparison)
__device__ __forceinline__ bool ne0(double x) { return (bits(x) & MAG) != 0; }
// fabs(x) > 0.0 (false for NaN)
__device__ __forceinline__ bool abs_gt0(double x) {
    const long long m = bits(x) & MAG;
    return m != 0 && m <= INF_BITS;
}

__device__ __forceinline__ double min(double a, double b) {
    if (isnan_(a)) return b;
    if (isnan_(b)) return a;
    return key(b) < key(a) ? b : a;
}
__device__ __forceinline__ double max(double a, double b) {
    if (isnan_(a)) return b;
    if (isnan_(b)) return a;
    return key(b) > key(a) ? b : a;
}

} // namespace ic
} // namespace ctsmg
