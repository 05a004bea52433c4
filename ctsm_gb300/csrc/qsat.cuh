// qsat.cuh -- QSat (src/biogeophys/QSatMod.F90:61-127): saturation vapour
// pressure and specific humidity over water (T >= tfrz) or ice by the
// module's 8th-order polynomials, shared by the canopy and bare-ground kernels.
#pragma once
#include <cuda_runtime.h>
#include "ctsm_device.cuh"

namespace ctsmg {

// QSatMod.F90:61-127
__device__ inline void qsat(double T, double p, double& qs, double& es, double* qsdT) {
    double td = fmin(100.0, fmax(-75.0, T - TFRZ));
    double esl;
    if (td >= 0.0)
        esl = 6.11213476 + td * (0.444007856 + td * (0.143064234e-01 + td * (0.264461437e-03 + td * (0.305903558e-05 +
              td * (0.196237241e-07 + td * (0.892344772e-10 + td * (-0.373208410e-12 + td * 0.209339997e-15)))))));
    else
        esl = 6.11123516 + td * (0.503109514 + td * (0.188369801e-01 + td * (0.420547422e-03 + td * (0.614396778e-05 +
              td * (0.602780717e-07 + td * (0.387940929e-09 + td * (0.149436277e-11 + td * 0.262655803e-14)))))));
    esl = esl * 100.0;
    const double vp = 1.0 / (p - 0.378 * esl);
    const double vp1 = 0.622 * vp;
    qs = esl * vp1;
    es = esl;
    if (qsdT) {
        double esdT;
        if (td >= 0.0)
            esdT = 0.444017302 + td * (0.286064092e-01 + td * (0.794683137e-03 + td * (0.121211669e-04 + td * (0.103354611e-06 +
                   td * (0.404125005e-09 + td * (-0.788037859e-12 + td * (-0.114596802e-13 + td * 0.381294516e-16)))))));
        else
            esdT = 0.503277922 + td * (0.377289173e-01 + td * (0.126801703e-02 + td * (0.249468427e-04 + td * (0.313703411e-06 +
                   td * (0.257180651e-08 + td * (0.133268878e-10 + td * (0.394116744e-13 + td * 0.498070196e-16)))))));
        esdT = esdT * 100.0;
        *qsdT = esdT * (vp1 * vp) * p;
    }
}

} // namespace ctsmg

