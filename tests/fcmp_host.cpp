// Host build of ctsm_gb300/csrc/fcmp.cuh for the tests: every comparison,
// min and max form against the host's IEEE comparisons and fmin / fmax, on
// the edge cases (signed zeros, subnormals, infinities, NaN of either sign,
// the literals the kernels compare against) and on n random pairs drawn by a
// xorshift generator from `seed` (random bit patterns, and values of
// physical magnitude).  Returns the number of disagreements.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include "fcmp.cuh"

using namespace ctsmg;

static uint64_t s_state;
static uint64_t next() { s_state ^= s_state << 13; s_state ^= s_state >> 7; s_state ^= s_state << 17; return s_state; }
static double from(uint64_t u) { double d; std::memcpy(&d, &u, 8); return d; }
static bool same(double a, double b) { return a == b || (std::isnan(a) && std::isnan(b)); }
// fmin / fmax as IEEE minNum / maxNum with quiet semantics for every NaN (a
// NaN operand yields the other one), which is what the device instructions do
static double fmin_q(double a, double b) { return std::isnan(a) ? b : std::isnan(b) ? a : (b < a ? b : a); }
static double fmax_q(double a, double b) { return std::isnan(a) ? b : std::isnan(b) ? a : (b > a ? b : a); }

static long long check_pair(double x, double y) {
    long long bad = 0;
    bad += ic::lt(x, y) != (x < y);
    bad += ic::le(x, y) != (x <= y);
    bad += ic::gt(x, y) != (x > y);
    bad += ic::ge(x, y) != (x >= y);
    bad += ic::eq(x, y) != (x == y);
    bad += ic::ne0(x) != (x != 0.0);
    bad += ic::abs_gt0(x) != (std::fabs(x) > 0.0);
    bad += ic::abs_ge(x, y) != (std::fabs(x) >= std::fabs(y));
    bad += !same(ic::min(x, y), fmin_q(x, y));
    bad += !same(ic::max(x, y), fmax_q(x, y));
    bad += ic::lt0(x) != (x < 0.0);
    bad += ic::le0(x) != (x <= 0.0);
    bad += ic::gt0(x) != (x > 0.0);
    bad += ic::ge0(x) != (x >= 0.0);
    bad += !same(ic::max0(x), fmax_q(x, 0.0));
    if (y > 0.0) {
        bad += ic::ltc(x, y) != (x < y);
        bad += ic::lec(x, y) != (x <= y);
        bad += ic::gtc(x, y) != (x > y);
        bad += ic::gec(x, y) != (x >= y);
        bad += !same(ic::minc(x, y), fmin_q(x, y));
        bad += !same(ic::maxc(x, y), fmax_q(x, y));
    } else if (y < 0.0) {
        bad += ic::ltn(x, y) != (x < y);
        bad += ic::gtn(x, y) != (x > y);
    }
    return bad;
}

extern "C" long long fcmp_check(long long n, unsigned long long seed) {
    const double inf = std::numeric_limits<double>::infinity();
    const double sp[] = {0.0, -0.0, 1.0, -1.0, inf, -inf, from(0x7ff8000000000000ull), from(0xfff8000000000000ull),
                         from(0x7ff0000000000001ull), from(0xfff0000000000001ull), 5e-324, -5e-324,
                         2.2250738585072014e-308, -2.2250738585072014e-308, 1.7976931348623157e308,
                         -1.7976931348623157e308, 273.15, std::nextafter(273.15, 400.0), std::nextafter(273.15, 0.0),
                         1e-6, 0.01, 0.1, 156.0, 1e-7, 10.0, 50.0, -0.01, -100.0, -1.574, -0.465, -6.661338147750939e-16};
    long long bad = 0;
    for (double x : sp)
        for (double y : sp) bad += check_pair(x, y);
    s_state = seed | 1;
    for (long long i = 0; i < n; ++i) {
        const uint64_t ra = next(), rb = next();
        double x, y;
        switch (i & 3) {
        case 0: x = from(ra); y = from(rb); break;                                   // any bit pattern
        case 1: x = from(ra); y = sp[rb % (sizeof(sp) / sizeof(sp[0]))]; break;      // against the literals
        case 2: x = (double)(int64_t)(ra >> 40) * 1e-3 - 8000.0; y = from(rb); break;
        default: x = (double)(int64_t)(ra >> 44) * 1e-2 - 400.0; y = (double)(int64_t)(rb >> 44) * 1e-2 - 400.0;
        }
        bad += check_pair(x, y);
    }
    return bad;
}
