// hydrology_kernels.cuh -- launcher of the water-table and drainage routines (internal C++ API).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "ctsm_gpu.h"

namespace ctsmg {

enum HydrologyRoutine { HYD_SAT_EXCESS = 0, HYD_PERCHED_WT, HYD_THETA_WT, HYD_PERCHED_LAT, HYD_SUBSURFACE_LAT, HYD_INFIL,
                        HYD_WATER_TABLE, HYD_DRAINAGE };

cudaError_t launch_hydrology(const ctsmg_hydrology_io& io, int begc, int n, const int32_t* d_filt, int which,
                             const ctsmg_soilhydrology_params& P, double dtime, cudaStream_t s);

} // namespace ctsmg
