// balance_kernels.cuh -- per-column water / soil-energy balance of a step.
#pragma once
#include <cuda_runtime.h>
#include "ctsm_device.cuh"

namespace ctsmg {
struct BalanceState {
    double* tssbef;        // [SS] t_soisno at the start of the step
    double* th2osfc_bef;   // (c)
    double* w_bef;         // (c)  column water at the start of the step (mm)
    double* errh2o;        // (c)  last step's water error (mm)
    double* errsoi;        // (c)  last step's soil energy error (W/m2)
    double* errh2o_max;    // (c)  max |errh2o| over steps >= skip_steps
    double* errsoi_max;    // (c)
    int* step;             // steps completed
    int skip_steps;
    int mf_lbc;            // 0: Zeng-Decker; else the moisture form's lower boundary condition
};
cudaError_t launch_prestep(const ctsmg_soiltemp_io& t, int ncol, const BalanceState& bs, cudaStream_t s);
cudaError_t launch_balance(const ctsmg_soilwater_io& w, const ctsmg_soiltemp_io& t, int ncol, double dtime,
                           const BalanceState& bs, cudaStream_t s);
} // namespace ctsmg
