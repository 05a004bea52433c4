// rootmoist_kernels.cuh -- launcher of the root moisture stress kernel (internal C++ API).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "ctsm_gpu.h"

namespace ctsmg {
// d_filtp: device copy of the 1-based patch filter, or NULL for begp .. begp+nfp-1.
cudaError_t launch_rootmoist(const ctsmg_rootmoist_io& io, const ctsmg_pftcon& pft, int begc, int begp, int nfp,
                             const int32_t* d_filtp, cudaStream_t s);
} // namespace ctsmg
