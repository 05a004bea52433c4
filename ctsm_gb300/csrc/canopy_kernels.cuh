// canopy_kernels.cuh -- launcher of the CanopyFluxes kernel (internal C++ API).
#pragma once
#include <cuda_runtime.h>
#include "ctsm_device.cuh"

namespace ctsmg {
struct CanopyArgs {
    ctsmg_canopy_io io;        // device pointers
    ctsmg_canopy_params par;
    ctsmg_pftcon pft;
    int method;                // 1 = Medlyn 2011, 0 = Ball-Berry 1987
    int itmax;                 // itmax_canopy_fluxes
    int begc, begp;
    // batched mode: keep displa / z0mv (SatellitePhenology inputs) unchanged
    // and start cgrnds / cgrndl from zero every step, as the driver does
    int engine;
    // optional per-patch Medlyn parameters (ensemble members); NULL = pftcon
    const double* medlynslope_p;
    const double* medlynintercept_p;
};
cudaError_t launch_canopy(const CanopyArgs& a, int nfilt, const int32_t* d_filt, double dtime, int* d_counter,
                          DevError* err, cudaStream_t s);
} // namespace ctsmg
