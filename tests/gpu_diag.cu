// gpu_diag.cu -- test-only library (not part of libctsm_gpu.so): the column
// kernels' device math beside CUDA's functions, for the GPU tests.
//   ctsmg_diag_powers(n, a, b, out): out[i] = pow(10, a[i]), out[n+i] = the
//     soil step's exp form of it, out[2n+i] = pow(tkwat, a[i]) * pow(tkice,
//     b[i]), out[3n+i] = the exp form of that product (4n doubles).
//   ctsmg_diag_fastmath(n, x, y, out): the table-driven log, log10, exp, pow
//     (rows 0-3) and CUDA's log, log10, exp, pow (rows 4-7) (8n doubles).
//   ctsmg_diag_crdiv(n, a, b, out): out[i] = a[i] / b[i] (CUDA), out[n+i] =
//     the shared-reciprocal quotient of cr_div.cuh, out[2n+i] = its
//     reciprocal RN(1/b[i]) (3n doubles).
//   ctsmg_diag_fcmp(n, a, b, out): the integer-pipe comparisons of fcmp.cuh
//     beside the FP64 ones -- rows 0-6 a<b, a<=b, a>b, a>=b, a==b, a!=0,
//     |a|>0 (IEEE), row 7 fmax(a, 0), rows 8-14 the same seven from
//     fcmp.cuh, row 15 ic::abs_ge(a, b), rows 16-19 fmin(a,b), fmax(a,b),
//     ic::min, ic::max, row 20 fm::i2d(i - n/2),
//     rows 21-24 ic::ltc, lec, gtc, gec (b > 0) or ltn, -, gtn, - (b < 0),
//     rows 25-28 ic::lt0, le0, gt0, ge0 of a, rows 29-31 ic::minc(a, b),
//     ic::maxc(a, b) (b > 0), ic::max0(a) (32n doubles).
// Host arrays in and out.  Built by tests/gpu_diag.py with nvcc for sm_103a.
#include <cuda_runtime.h>
#include <cstdint>
#include "ctsm_gpu.h"
#include "ctsm_device.cuh"
#include "soil_math.cuh"
#include "cr_div.cuh"
#include "fcmp.cuh"

static int32_t diag_fail(cudaError_t e) { return e == cudaSuccess ? 0 : CTSMG_E_CUDA; }

namespace ctsmg {
__global__ void diag_powers_kernel(int n, const double* __restrict__ a, const double* __restrict__ b,
                                   double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = pow(10.0, a[i]);
    out[n + i] = pow10_dd(a[i]);
    out[2 * (size_t)n + i] = pow(TKWAT, a[i]) * pow(TKICE, b[i]);
    out[3 * (size_t)n + i] = tkwat_tkice_pow(a[i], b[i]);
}
__global__ void diag_fastmath_kernel(int n, const double* __restrict__ x, const double* __restrict__ y,
                                     double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t N = (size_t)n;
    out[i] = fm::log(x[i]);
    out[N + i] = fm::log10(x[i]);
    out[2 * N + i] = fm::exp(y[i]);
    out[3 * N + i] = fm::pow(x[i], y[i]);
    out[4 * N + i] = log(x[i]);
    out[5 * N + i] = log10(x[i]);
    out[6 * N + i] = exp(y[i]);
    out[7 * N + i] = pow(x[i], y[i]);
}
} // namespace ctsmg

extern "C" int32_t ctsmg_diag_fastmath(int32_t n, const double* x, const double* y, double* out) {
    using namespace ctsmg;
    if (n <= 0 || !x || !y || !out) return CTSMG_E_ARG;
    double* d = nullptr;
    const size_t nb = (size_t)n * 8;
    cudaError_t e = cudaMalloc(&d, 10 * nb);
    if (e == cudaSuccess) e = cudaMemcpy(d, x, nb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d + n, y, nb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        diag_fastmath_kernel<<<(n + 127) / 128, 128>>>(n, d, d + n, d + 2 * (size_t)n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, d + 2 * (size_t)n, 8 * nb, cudaMemcpyDeviceToHost);
    if (d) cudaFree(d);
    return diag_fail(e);
}

extern "C" int32_t ctsmg_diag_powers(int32_t n, const double* a, const double* b, double* out) {
    using namespace ctsmg;
    if (n <= 0 || !a || !b || !out) return CTSMG_E_ARG;
    double* d = nullptr;
    const size_t nb = (size_t)n * 8;
    cudaError_t e = cudaMalloc(&d, 6 * nb);
    if (e == cudaSuccess) e = cudaMemcpy(d, a, nb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d + n, b, nb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        diag_powers_kernel<<<(n + 127) / 128, 128>>>(n, d, d + n, d + 2 * (size_t)n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, d + 2 * (size_t)n, 4 * nb, cudaMemcpyDeviceToHost);
    if (d) cudaFree(d);
    return diag_fail(e);
}

namespace ctsmg {
__global__ void diag_crdiv_kernel(int n, const double* __restrict__ a, const double* __restrict__ b,
                                  double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Recip R = recip(b[i]);
    out[i] = a[i] / b[i];
    out[n + i] = divr(a[i], R);
    out[2 * (size_t)n + i] = R.y;
}
} // namespace ctsmg

extern "C" int32_t ctsmg_diag_crdiv(int32_t n, const double* a, const double* b, double* out) {
    using namespace ctsmg;
    if (n <= 0 || !a || !b || !out) return CTSMG_E_ARG;
    double* d = nullptr;
    const size_t nb = (size_t)n * 8;
    cudaError_t e = cudaMalloc(&d, 5 * nb);
    if (e == cudaSuccess) e = cudaMemcpy(d, a, nb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d + n, b, nb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        diag_crdiv_kernel<<<(n + 127) / 128, 128>>>(n, d, d + n, d + 2 * (size_t)n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, d + 2 * (size_t)n, 3 * nb, cudaMemcpyDeviceToHost);
    if (d) cudaFree(d);
    return diag_fail(e);
}

namespace ctsmg {
__global__ void diag_fcmp_kernel(int n, const double* __restrict__ a, const double* __restrict__ b,
                                 double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = a[i], y = b[i];
    auto put = [&](int row, double v) { out[(size_t)row * n + i] = v; };
    put(0, x < y); put(1, x <= y); put(2, x > y); put(3, x >= y); put(4, x == y); put(5, x != 0.0);
    put(6, fabs(x) > 0.0); put(7, fmax(x, 0.0));
    put(8, ic::lt(x, y)); put(9, ic::le(x, y)); put(10, ic::gt(x, y)); put(11, ic::ge(x, y));
    put(12, ic::eq(x, y)); put(13, ic::ne0(x)); put(14, ic::abs_gt0(x)); put(15, ic::abs_ge(x, y));
    put(16, fmin(x, y)); put(17, fmax(x, y)); put(18, ic::min(x, y)); put(19, ic::max(x, y));
    put(20, fm::i2d(i - n / 2));
    const bool pos = y > 0.0;
    put(21, pos ? ic::ltc(x, y) : ic::ltn(x, y)); put(22, pos ? ic::lec(x, y) : 0.0);
    put(23, pos ? ic::gtc(x, y) : ic::gtn(x, y)); put(24, pos ? ic::gec(x, y) : 0.0);
    put(25, ic::lt0(x)); put(26, ic::le0(x)); put(27, ic::gt0(x)); put(28, ic::ge0(x));
    put(29, pos ? ic::minc(x, y) : 0.0); put(30, pos ? ic::maxc(x, y) : 0.0); put(31, ic::max0(x));
}
} // namespace ctsmg

extern "C" int32_t ctsmg_diag_fcmp(int32_t n, const double* a, const double* b, double* out) {
    using namespace ctsmg;
    if (n <= 0 || !a || !b || !out) return CTSMG_E_ARG;
    double* d = nullptr;
    const size_t nb = (size_t)n * 8;
    cudaError_t e = cudaMalloc(&d, 34 * nb);
    if (e == cudaSuccess) e = cudaMemcpy(d, a, nb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d + n, b, nb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        diag_fcmp_kernel<<<(n + 127) / 128, 128>>>(n, d, d + n, d + 2 * (size_t)n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, d + 2 * (size_t)n, 32 * nb, cudaMemcpyDeviceToHost);
    if (d) cudaFree(d);
    return diag_fail(e);
}
