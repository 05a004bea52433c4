// soilfluxes_kernels.cu -- SoilFluxes (src/biogeophys/SoilFluxesMod.F90) for
// natural-vegetation patches: one thread per patch of filter_nolakep, then the
// filtered p2c of errsoi over filter_nolakec (src/main/subgridAveMod.F90:292-320).
#include <cuda_runtime.h>
#include <cstdint>
#include "ctsm_device.cuh"
#include "soilfluxes_device.cuh"
#include "soilfluxes_kernels.cuh"

namespace ctsmg {

__global__ void soilfluxes_patch_kernel(ctsmg_soilfluxes_io io, int begc, int begp, int nfp,
                                        const int32_t* __restrict__ filtp, double dtime) {
    const int fp = blockIdx.x * blockDim.x + threadIdx.x;
    if (fp >= nfp) return;
    const int p = filtp[fp] - begp;
    soilfluxes_patch(io, p, io.patch_column[p] - begc, dtime);
}

__global__ void soilfluxes_p2c_kernel(ctsmg_soilfluxes_io io, int begc, int begp, int nfc,
                                      const int32_t* __restrict__ filtc) {
    const int fc = blockIdx.x * blockDim.x + threadIdx.x;
    if (fc >= nfc) return;
    soilfluxes_p2c(io, filtc[fc] - begc, begp);
}

cudaError_t launch_soilfluxes(const ctsmg_soilfluxes_io& io, int begc, int begp, int nfc, const int32_t* d_filtc,
                              int nfp, const int32_t* d_filtp, double dtime, cudaStream_t s) {
    if (nfp > 0) soilfluxes_patch_kernel<<<(nfp + 127) / 128, 128, 0, s>>>(io, begc, begp, nfp, d_filtp, dtime);
    if (nfc > 0) soilfluxes_p2c_kernel<<<(nfc + 127) / 128, 128, 0, s>>>(io, begc, begp, nfc, d_filtc);
    return cudaGetLastError();
}

} // namespace ctsmg
