// surface_resistance_kernels.cu -- the drop-in kernel of calc_soilevap_resis
// (src/biogeophys/SurfaceResistanceMod.F90:190-227): one thread per column.
#include <cuda_runtime.h>
#include <cstdint>
#include "surface_resistance.cuh"

namespace ctsmg {

__global__ void __launch_bounds__(128)
soilevap_resis_kernel(ctsmg_soilresis_io io, int begc, int nfilt, const int32_t* __restrict__ filt, SoilResisArgs a) {
    const int fc = blockIdx.x * blockDim.x + threadIdx.x;
    if (fc >= nfilt) return;
    soilevap_resis_column(io, (filt ? filt[fc] : fc + begc) - begc, a);
}

cudaError_t launch_soilevap_resis(const ctsmg_soilresis_io& io, int begc, int nfilt, const int32_t* d_filt,
                                  const SoilResisArgs& a, cudaStream_t s) {
    if (nfilt <= 0) return cudaSuccess;
    soilevap_resis_kernel<<<(nfilt + 127) / 128, 128, 0, s>>>(io, begc, nfilt, d_filt, a);
    return cudaGetLastError();
}

} // namespace ctsmg
