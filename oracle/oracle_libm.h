// oracle_libm.h -- libm calls of the oracle, with the optional per-call noise
// used by the conditioning tests (off unless oracle_set_libm_noise is called).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace oracle_libm {
extern int g_noise_ulps;
extern uint64_t g_noise_seed;
inline uint64_t mix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
inline double noisy(double r, double a, double b) {
    if (g_noise_ulps <= 0) return r;
    uint64_t ua, ub;
    std::memcpy(&ua, &a, 8); std::memcpy(&ub, &b, 8);
    uint64_t h = mix64(ua ^ mix64(ub ^ g_noise_seed));
    int k = (int)(h % (uint64_t)(2 * g_noise_ulps + 1)) - g_noise_ulps;
    return r * (1.0 + k * 2.220446049250313e-16);
}
inline double o_pow(double x, double y) { return noisy(std::pow(x, y), x, y); }
inline double o_log10(double x) { return noisy(std::log10(x), x, 1.0); }
inline double o_exp(double x) { return noisy(std::exp(x), x, 2.0); }
inline double o_log(double x) { return noisy(std::log(x), x, 3.0); }
inline double o_atan(double x) { return noisy(std::atan(x), x, 4.0); }
} // namespace oracle_libm
