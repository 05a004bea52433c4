// hydrology_kernels.cu -- drop-in kernels of the water-table and drainage
// routines around SoilWater (one thread per column of filter_hydrologyc);
// the per-column bodies are in hydrology_device.cuh.
#include <cuda_runtime.h>
#include <cstdint>
#include "hydrology_device.cuh"
#include "hydrology_kernels.cuh"

namespace ctsmg {

__global__ void __launch_bounds__(128)
hydrology_kernel(ctsmg_hydrology_io io, int begc, int n, const int32_t* __restrict__ filt, int which,
                 ctsmg_soilhydrology_params P, double dtime) {
    const int fc = blockIdx.x * blockDim.x + threadIdx.x;
    if (fc >= n) return;
    const int c = filt[fc] - begc;
    switch (which) {
        case HYD_SAT_EXCESS: hydro::saturated_excess_runoff(io, c, P.fff); break;
        case HYD_PERCHED_WT: hydro::perched_water_table(io, c); break;
        case HYD_THETA_WT: hydro::theta_based_water_table(io, c); break;
        case HYD_PERCHED_LAT: hydro::perched_lateral_flow(io, c, P, dtime); break;
        case HYD_INFIL: hydro::infiltration_chain(io, c, P, dtime); break;
        case HYD_WATER_TABLE: hydro::water_table(io, c, P, dtime); break;
        case HYD_DRAINAGE: hydro::drainage(io, c, P, dtime); break;
        default: hydro::subsurface_lateral_flow(io, c, P, dtime); break;
    }
}

cudaError_t launch_hydrology(const ctsmg_hydrology_io& io, int begc, int n, const int32_t* d_filt, int which,
                             const ctsmg_soilhydrology_params& P, double dtime, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    hydrology_kernel<<<(n + 127) / 128, 128, 0, s>>>(io, begc, n, d_filt, which, P, dtime);
    return cudaGetLastError();
}

} // namespace ctsmg
