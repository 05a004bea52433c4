// soil_kernels.cuh -- launchers of the soil-path kernels (internal C++ API).
#pragma once
#include <cuda_runtime.h>
#include "ctsm_device.cuh"

namespace ctsmg {
// rows of heat-system scratch per column (6 doubles per row)
constexpr int SOILTEMP_WS_DOUBLES_PER_COL = 6 * NROW_MAX;

cudaError_t launch_soilwater(const ctsmg_soilwater_io& io, int begc, int nfilt, const int32_t* d_filt,
                             double e_ice, double dtime, cudaStream_t s);
cudaError_t launch_soiltemp(const ctsmg_soiltemp_io& io, int begc, int begp, int nfilt, const int32_t* d_filt,
                            double dtime, int snow_method, double* ws, int ws_ld, DevError* err, cudaStream_t s);
// Columns one launch of the drop-in kernel keeps resident on the whole GPU
// at once (SMs x resident blocks x block size): the size of a chunk of a
// pipelined drop-in call that fills the GPU without a partial second wave.
int soiltemp_wave_columns();
// What the fused soil step does beside the heat solve: water = 1 runs the
// Zeng-Decker SoilWater inside (0: the caller runs the moisture form in its
// own kernel), flexcn = 1 applies the use_flexibleCN fix after it, refresh = 1
// refreshes h2osoi_vol at the end.
struct SoilStepFlags {
    int water = 1, flexcn = 0, refresh = 1;
};
cudaError_t launch_soilstep(const ctsmg_soilwater_io& wio, const ctsmg_soiltemp_io& tio, int ncol,
                            double e_ice, double dtime, int snow_method, double* ws, int ws_ld,
                            DevError* err, cudaStream_t s, int block, int order = 0,
                            const int32_t* filt = nullptr, const ctsmg_soilfluxes_io* sf = nullptr,
                            SoilStepFlags fl = SoilStepFlags());
struct HydroStepArgs;
// The Zeng-Decker SoilWater of a resident step in its own kernel (with the
// aquifer-layer hydrology when hy is given).
cudaError_t launch_zd09_step(const ctsmg_soilwater_io& io, int ncol, double e_ice, double dtime, int flexcn,
                             int refresh, const int32_t* d_filt, cudaStream_t s, const HydroStepArgs* hy);
cudaError_t launch_rootsink_dropin(const ctsmg_rootsink_io& io, int begc, int begp, int nfilt, const int32_t* d_filt,
                                   cudaStream_t s);
cudaError_t launch_rootsink(const int32_t* col_patchi, const int32_t* col_npatches, const double* wtcol,
                            const double* qflx_tran_veg, const double* rootr, int ldp, double* qflx_rootsoi,
                            int ncol, cudaStream_t s, int ldc = 0, const int32_t* filt = nullptr);
cudaError_t launch_permute(void* dst, const void* src, const int32_t* perm, int ncol, int nlev, int esize,
                           int scatter, cudaStream_t s);
} // namespace ctsmg
