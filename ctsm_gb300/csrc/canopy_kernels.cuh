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
// Device bytes of the per-patch iteration records of a call over nfilt patches.
size_t canopy_ws_bytes(int nfilt);
size_t canopy_ws_bytes_per_patch();
// ws: canopy_ws_bytes(nfilt) bytes of device memory, 8-byte aligned.
cudaError_t launch_canopy(const CanopyArgs& a, int nfilt, const int32_t* d_filt, double dtime, int* d_counter,
                          DevError* err, double* ws, cudaStream_t s);
} // namespace ctsmg
