// rootmoist_kernels.cu -- the root moisture stress CanopyFluxes computes before
// its iteration (src/biogeophys/CanopyFluxesMod.F90:709, 833-895): effective
// porosity and volumetric liquid water of soil levels 1..nlevgrnd
// (SoilMoistStressMod.F90:70-114, 171-217) and calc_root_moist_stress_clm45default
// (:312-435) with the Clapp-Hornberger suction
// (SoilWaterRetentionCurveClappHornberg1978Mod.F90:87-125).  One thread per
// patch of the filter; patches of one column write identical porosity values.
#include <cuda_runtime.h>
#include <cstdint>
#include "ctsm_device.cuh"
#include "fastmath.cuh"
#include "rootmoist_kernels.cuh"

namespace ctsmg {

__global__ void rootmoist_kernel(ctsmg_rootmoist_io io, ctsmg_pftcon pft, int begc, int begp, int nfp,
                                 const int32_t* __restrict__ filtp) {
    const int fp = blockIdx.x * blockDim.x + threadIdx.x;
    if (fp >= nfp) return;
    const int p = (filtp ? filtp[fp] : fp + begp) - begp;
    const int c = io.patch_column[p] - begc;
    const int ldc = io.ldc, ldp = io.ldp, it = io.itype[p];
    const double smpso = pft.smpso[it], smpsc = pft.smpsc[it];
    double btran = 0.0;                                     // btran0 (:709)
#pragma unroll 1
    for (int j = 1; j <= NLEVGRND; ++j) {
        const size_t ss = c + (size_t)(j - LS) * ldc, g = c + (size_t)(j - 1) * ldc, pg = p + (size_t)(j - 1) * ldp;
        const double ws = io.watsat[g], dz = io.dz[ss];
        const double vol_ice = fmin(ws, io.h2osoi_ice[ss] / (DENICE * dz));
        const double eff = ws - vol_ice;
        const double liqvol = fmin(eff, io.h2osoi_liq[ss] / (dz * DENH2O));
        io.eff_porosity[g] = eff;
        io.h2osoi_liqvol[g] = liqvol;
        if (liqvol <= 0.0 || io.t_soisno[ss] <= TFRZ - 2.0) {
            io.rootr[pg] = 0.0;
        } else {
            const double s_node = fmax(liqvol / eff, 0.01);
            double smp = -io.sucsat[g] * fm::pow(s_node, -io.bsw[g]);
            smp = fmax(smpsc, smp);
            const double rr = fmin((eff / ws) * (smp - smpsc) / (smpso - smpsc), 1.0);
            io.rresis[pg] = rr;
            const double root = io.rootfr[pg] * rr;
            io.rootr[pg] = root;
            btran = btran + fmax(root, 0.0);
        }
    }
    io.btran[p] = btran;
#pragma unroll 1
    for (int j = 1; j <= NLEVGRND; ++j) {
        const size_t pg = p + (size_t)(j - 1) * ldp;
        io.rootr[pg] = (btran > 0.0) ? io.rootr[pg] / btran : 0.0;
    }
}

cudaError_t launch_rootmoist(const ctsmg_rootmoist_io& io, const ctsmg_pftcon& pft, int begc, int begp, int nfp,
                             const int32_t* d_filtp, cudaStream_t s) {
    if (nfp <= 0) return cudaSuccess;
    rootmoist_kernel<<<(nfp + 127) / 128, 128, 0, s>>>(io, pft, begc, begp, nfp, d_filtp);
    return cudaGetLastError();
}

} // namespace ctsmg
