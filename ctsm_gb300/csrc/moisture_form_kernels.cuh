// moisture_form_kernels.cuh -- launchers of SoilWater's moisture form and of
// the use_flexibleCN fix (internal C++ API).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "ctsm_gpu.h"
#include "ctsm_device.cuh"

namespace ctsmg {

struct MoistureFormArgs {
    double e_ice, dtime, dtmin, verySmall, xTolerUpper, xTolerLower;
    int lower_bc;        // 1 bc_flux, 2 bc_zero_flux, 3 bc_waterTable
    int expensive;       // flux_calculation == expensive
    int max_trials;      // bound on the sub-step loop (never reached by the reference's rule)
};

// Trials the halving/doubling rule can take at most: every accepted sub-step
// is at least dtmin long (or the remainder) and is preceded by at most one
// rejected doubling, after the initial halvings from dtime down to dtmin.
inline int moisture_form_max_trials(double dtime, double dtmin) {
    double n = dtime / (dtmin > 0.0 ? dtmin : dtime);
    if (n > 1.0e6) n = 1.0e6;
    return 2 * (int)n + 128;
}


// d_filt: device copy of the 1-based column filter, or NULL for begc .. begc+nfilt-1.
cudaError_t launch_moisture_form(const ctsmg_soilwater_io& io, int begc, int nfilt, const int32_t* d_filt,
                                 const MoistureFormArgs& P, DevError* err, cudaStream_t s, int* d_counter);
// The default hydrology around SoilWater in the resident step: per-column
// baseflow_scalar / fff override the parameters where given.
struct HydroStepArgs {
    ctsmg_hydrology_io io;
    ctsmg_soilhydrology_params par;
    const double* baseflow_scalar_c;
    const double* fff_c;
};

// The resident step's work order for the persistent sub-step kernel: every
// step the filter positions are bucketed by the sub-step count their column
// took the step before (1, 2, 3-4, 5-8, 9-16, more) and by its bedrock depth
// (the length of each trial's level loops), both descending, so the lanes of
// a warp run level loops of one length, finish their sub-step loops together
// and the longest columns start first.  The scratch holds the work counter,
// the bucket histogram and fill counters, each position's bucket and the
// order itself.
constexpr int MF_NCLS = 6;
constexpr int MF_NKEY = MF_NCLS * NLEVSOI;
constexpr int MF_WORK_HEAD = 32 + 2 * MF_NKEY;       // ints before the per-position arrays
inline size_t mf_work_bytes(int ncol) { return ((size_t)MF_WORK_HEAD + 2 * (size_t)(ncol > 0 ? ncol : 0)) * sizeof(int); }
// With the work order, the sub-step kernel runs on a compact copy of the
// components it uses, moved into the order (and the written ones back): the
// workspace bytes for ncol columns.
constexpr int MF_MOVES = 24;
size_t mf_compact_bytes(int ncol);

// Resident-step form over positions 0..ncol-1 (or the 1-based position
// filter); hy = NULL leaves the hydrology out.
// d_work: device scratch, one int (the persistent kernel's work counter) or,
// with sorted, mf_work_bytes(ncol) for the bucketed work order; d_compact
// (with sorted; may be NULL) mf_compact_bytes(ncol) of workspace for the
// compact copy.
cudaError_t launch_mf_step(const ctsmg_soilwater_io& io, int ncol, const MoistureFormArgs& P, int flexcn, int refresh,
                           DevError* err, const int32_t* d_filt, cudaStream_t s, int* d_work,
                           const HydroStepArgs* hy = nullptr, bool sorted = false, void* d_compact = nullptr);
cudaError_t launch_set_soil_water_fractions(const ctsmg_soilwater_io& io, int begc, int nfilt, const int32_t* d_filt,
                                            cudaStream_t s);
cudaError_t launch_flexcn(const ctsmg_soilwater_io& io, int begc, int nfilt, const int32_t* d_filt, cudaStream_t s);

} // namespace ctsmg
