// moisture_form_device.cuh -- per-column device steps around SoilWater shared
// by the moisture-form kernels and the fused resident soil step.
#pragma once
#include <cuda_runtime.h>
#include "ctsm_gpu.h"
#include "ctsm_device.cuh"
#include "fcmp.cuh"

namespace ctsmg {

// SetSoilWaterFractions (src/biogeophys/SoilHydrologyMod.F90:236-249), no
// excess ice (dz_ext = dz): eff_porosity and icefrac on levels 1..nlevsoi.
__device__ __forceinline__ void set_soil_water_fractions(const ctsmg_soilwater_io& io, int c) {
    const int ld = io.ldc;
#pragma unroll 1
    for (int j = 1; j <= NLEVSOI; ++j) {
        const size_t ix = c + (size_t)(j - LS) * ld, g = c + (size_t)(j - 1) * ld;
        const double ws = io.watsat[g];
        const double dz_ext = io.dz[ix] + 0.0 / DENICE;
        const double a = io.h2osoi_ice[ix] + 0.0, q = a / (dz_ext * DENICE);
        const double vol_ice = ic::lt(q, ws) ? q : ws;
        const double ep = ws - vol_ice;
        ((double*)io.eff_porosity)[g] = ic::gtc(ep, 0.01) ? ep : 0.01;
        const double f = vol_ice / ws;
        io.icefrac[g] = ic::ltc(f, 1.0) ? f : 1.0;
    }
}

// SoilWater's use_flexibleCN fix (src/biogeophys/SoilWaterMovementMod.F90:331-368).
__device__ __forceinline__ void flexcn_column(const ctsmg_soilwater_io& io, int c) {
    const int ld = io.ldc;
    const double watmin = 0.001;
    double* liq = io.h2osoi_liq;
    double carry = liq[c + (size_t)(1 - LS) * ld];
#pragma unroll 1
    for (int j = 1; j <= NLEVSOI - 1; ++j) {
        const size_t ix = c + (size_t)(j - LS) * ld, ixn = ix + ld;
        const double xs = ic::lt0(carry) ? watmin - carry : 0.0;
        liq[ix] = carry + xs;
        carry = liq[ixn] - xs;
        liq[ixn] = carry;
    }
    const size_t ib = c + (size_t)(NLEVSOI - LS) * ld;
    const double xs = ic::ltc(carry, watmin) ? watmin - carry : 0.0;
    liq[ib] = carry + xs;
    io.wa[c] = io.wa[c] - xs;
#pragma unroll 1
    for (int j = 1; j <= NLEVSOI; ++j) {
        const size_t ix = c + (size_t)(j - LS) * ld;
        const double dz = io.dz[ix];
        ((double*)io.h2osoi_vol)[c + (size_t)(j - 1) * ld] = liq[ix] / (dz * DENH2O) + io.h2osoi_ice[ix] / (dz * DENICE);
    }
}

// h2osoi_vol = liq/(dz denh2o) + ice/(dz denice), levels 1..nlevsoi
// (HydrologyNoDrainageMod.F90:580,590).
__device__ __forceinline__ void refresh_h2osoi_vol(const ctsmg_soilwater_io& io, int c) {
    const int ld = io.ldc;
#pragma unroll 1
    for (int j = 1; j <= NLEVSOI; ++j) {
        const size_t ix = c + (size_t)(j - LS) * ld;
        const double dz = io.dz[ix];
        ((double*)io.h2osoi_vol)[c + (size_t)(j - 1) * ld] =
            io.h2osoi_liq[ix] / (dz * DENH2O) + io.h2osoi_ice[ix] / (dz * DENICE);
    }
}

} // namespace ctsmg
