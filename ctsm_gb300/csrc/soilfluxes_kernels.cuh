// soilfluxes_kernels.cuh -- launcher of the SoilFluxes kernels (internal C++ API).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "ctsm_gpu.h"

namespace ctsmg {
// d_filtc / d_filtp: device copies of filter_nolakec / filter_nolakep (1-based).
cudaError_t launch_soilfluxes(const ctsmg_soilfluxes_io& io, int begc, int begp, int nfc, const int32_t* d_filtc,
                              int nfp, const int32_t* d_filtp, double dtime, cudaStream_t s);
} // namespace ctsmg
