// ctsm_device.cuh -- constants and small device helpers shared by the kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "ctsm_gpu.h"

namespace ctsmg {

// physical constants: tools/mksurfdata_esmf/src/shr_const_mod.F90:14-56,
// src/main/clm_varcon.F90:48-121
constexpr double TFRZ = 273.15;
constexpr double GRAV = 9.80616;
constexpr double SB = 5.67e-8;
constexpr double DENH2O = 1.000e3;
constexpr double DENICE = 0.917e3;
constexpr double CPLIQ = 4.188e3;
constexpr double CPICE = 2.11727e3;
constexpr double HFUS = 3.337e5;
constexpr double TKAIR = 0.023;
constexpr double TKICE = 2.290;
constexpr double TKWAT = 0.57;
constexpr double CAPR = 0.34;
constexpr double CNFAC = 0.5;
constexpr double THK_BEDROCK = 3.0;
constexpr double CSOL_BEDROCK = 2.0e6;
constexpr double THIN_SFCLAYER = 1.0e-6;
constexpr double CTSMG_PI = 3.14159265358979323846;     // SHR_CONST_PI

constexpr int NLEVSNO = CTSMG_NLEVSNO;
constexpr int NLEVSOI = CTSMG_NLEVSOI;
constexpr int NLEVGRND = CTSMG_NLEVGRND;
constexpr int LS = -NLEVSNO + 1;                    // lowest snow level
constexpr int NROW_MAX = NLEVSNO + NLEVGRND + 1;    // heat-system rows -nlevsno..nlevgrnd

// single-precision literals of the reference, promoted
__host__ __device__ constexpr double sp(float x) { return (double)x; }

// device error record: the first failing filter index wins (atomicMin on a
// key with the filter index in the high word)
struct DevError {
    unsigned long long key;   // (fc << 32) | (level + 1024) << 8 | code ; ~0ull = none
};

__device__ __forceinline__ void report_error(DevError* e, int fc, int level, int code) {
    unsigned long long k = ((unsigned long long)(unsigned)fc << 32) |
                           ((unsigned long long)(unsigned)(level + 1024) << 8) |
                           (unsigned long long)(code & 0xff);
    atomicMin(&e->key, k);
}

// Column-array accessors: element (c, j) of a field whose Fortran lower bound
// is lb sits at base[c + (j - lb) * ld].
template <typename T>
struct Col {
    T* b; int ld;
    __device__ __forceinline__ T& at(int c, int j, int lb) const { return b[c + (size_t)(j - lb) * ld]; }
};

} // namespace ctsmg
