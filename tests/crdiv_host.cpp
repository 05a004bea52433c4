// Host build of ctsm_gb300/csrc/cr_div.cuh for the tests: every quotient of
// the shared-reciprocal form against the IEEE division, on n pairs (a, b)
// drawn by a xorshift generator from `seed` with the distributions named by
// `mode`.  Returns the number of pairs whose bits differ.  Built with
// -ffp-contract=off.
#include <cstdint>
#include <cstring>
#include "cr_div.cuh"

static uint64_t s_state;
static uint64_t next() { s_state ^= s_state << 13; s_state ^= s_state >> 7; s_state ^= s_state << 17; return s_state; }
static double from(uint64_t u) { double d; std::memcpy(&d, &u, 8); return d; }

extern "C" long long crdiv_check(long long n, unsigned long long seed, int mode) {
    s_state = seed | 1;
    long long bad = 0;
    for (long long i = 0; i < n; ++i) {
        const uint64_t ra = next(), rb = next();
        double a, b;
        if (mode == 0) {          // random significands, exponents over the whole double range
            a = from(ra & 0xffffffffffffffffull);
            b = from(rb & 0x7fffffffffffffffull);
        } else if (mode == 1) {   // physical magnitudes: exponents within 2^-40 .. 2^40
            a = from((ra & 0x800fffffffffffffull) | ((uint64_t)(1023 - 40 + (ra >> 56) % 81) << 52));
            b = from((rb & 0x000fffffffffffffull) | ((uint64_t)(1023 - 40 + (rb >> 56) % 81) << 52));
        } else if (mode == 2) {   // divisors with all-ones or nearly all-ones significands
            a = from((ra & 0x800fffffffffffffull) | ((uint64_t)(1023 - 20 + (ra >> 56) % 41) << 52));
            b = from((0x000fffffffffffffull ^ (rb & 0x3f)) | ((uint64_t)(1023 - 20 + (rb >> 56) % 41) << 52));
        } else {                  // quotients near rounding midpoints: a = b * m with m a midpoint +- a few ulp
            b = from((rb & 0x000fffffffffffffull) | (1023ull << 52));
            const double m = from(((ra & 0x000ffffffffffffeull) | 1ull | (1023ull << 52)));  // odd significand
            const double h = from((ra & 0x000fffffffffffffull) | (1023ull << 52));
            (void)h;
            a = b * (m + from(0x3ca0000000000000ull) * (double)((int)(ra >> 60) - 8));       // +- 8 * 2^-53
        }
        const ctsmg::Recip R = ctsmg::recip(b);
        const double q1 = a / b, q2 = ctsmg::divr(a, R);
        uint64_t u1, u2;
        std::memcpy(&u1, &q1, 8);
        std::memcpy(&u2, &q2, 8);
        if (u1 != u2 && !(q1 != q1 && q2 != q2)) ++bad;
    }
    return bad;
}
