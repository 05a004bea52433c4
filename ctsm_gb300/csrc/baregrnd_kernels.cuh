// baregrnd_kernels.cuh -- launcher of BareGroundFluxes (internal C++ API).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "ctsm_gpu.h"

namespace ctsmg {

struct BareArgs {
    double a_coef, a_exp, wind_min, zetamaxstable;
    int soil_resis_method;       // 1 sl_14 (soilresis), 0 leepielke_1992 (soilbeta)
};

// d_filt: device copy of the 1-based patch filter; d_last: ncol ints of scratch.
cudaError_t launch_baregrnd(const ctsmg_baregrnd_io& io, int begc, int begp, int nfp, const int32_t* d_filt,
                            const BareArgs& a, int* d_last, int ncol, cudaStream_t s);

} // namespace ctsmg
