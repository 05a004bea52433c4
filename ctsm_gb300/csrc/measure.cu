// measure.cu -- FP64 pipe peak of the current GPU, measured with a DFMA loop
// (8 independent chains per thread, every SM fully occupied).  Used as the
// denominator of the FP64 roofline fraction.
#include <cuda_runtime.h>
#include <cstdint>
#include "ctsm_gpu.h"

namespace {
__global__ void dfma_loop(double* out, int iters, double a, double b) {
    double x0 = threadIdx.x * 1e-9, x1 = x0 + 1e-3, x2 = x0 + 2e-3, x3 = x0 + 3e-3;
    double x4 = x0 + 4e-3, x5 = x0 + 5e-3, x6 = x0 + 6e-3, x7 = x0 + 7e-3;
#pragma unroll 1
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
            x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
        }
    }
    double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 12345.678) out[0] = s;   // keeps the chains live
}

// The same loop with only the first `active` lanes of each warp running it.
__global__ void dfma_loop_lanes(double* out, int iters, double a, double b, int active) {
    if ((int)(threadIdx.x & 31) >= active) return;
    double x0 = threadIdx.x * 1e-9, x1 = x0 + 1e-3, x2 = x0 + 2e-3, x3 = x0 + 3e-3;
    double x4 = x0 + 4e-3, x5 = x0 + 5e-3, x6 = x0 + 6e-3, x7 = x0 + 7e-3;
#pragma unroll 1
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
            x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
        }
    }
    double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 12345.678) out[0] = s;
}
// A chain of FP64 divisions (8 independent chains per thread) on the first
// `active` lanes of each warp.
__global__ void ddiv_loop_lanes(double* out, int iters, double a, int active) {
    if ((int)(threadIdx.x & 31) >= active) return;
    double x0 = 1.0 + threadIdx.x * 1e-9, x1 = x0 + 1e-3, x2 = x0 + 2e-3, x3 = x0 + 3e-3;
    double x4 = x0 + 4e-3, x5 = x0 + 5e-3, x6 = x0 + 6e-3, x7 = x0 + 7e-3;
#pragma unroll 1
    for (int i = 0; i < iters; ++i) {
        x0 = a / (x0 + 1.5); x1 = a / (x1 + 1.5); x2 = a / (x2 + 1.5); x3 = a / (x3 + 1.5);
        x4 = a / (x4 + 1.5); x5 = a / (x5 + 1.5); x6 = a / (x6 + 1.5); x7 = a / (x7 + 1.5);
    }
    double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 12345.678) out[0] = s;
}
} // namespace

// Milliseconds of ddiv_loop_lanes (256 x 8 divisions per thread, 8 blocks of
// 256 threads per SM) with the first active_lanes lanes of each warp active.
extern "C" int32_t ctsmg_measure_fp64_div_lane_cost(int32_t active_lanes, float* ms_out) {
    if (!ms_out || active_lanes < 1 || active_lanes > 32) return CTSMG_E_ARG;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return CTSMG_E_CUDA;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return CTSMG_E_CUDA;
    double* d = nullptr;
    if (cudaMalloc(&d, 8) != cudaSuccess) return CTSMG_E_CUDA;
    const int threads = 256, blocks = nsm * 8, iters = 256;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    ddiv_loop_lanes<<<blocks, threads>>>(d, 8, 2.0, active_lanes);
    cudaEventRecord(e0);
    ddiv_loop_lanes<<<blocks, threads>>>(d, iters, 2.0, active_lanes);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    if (err != cudaSuccess || ms <= 0.f) return CTSMG_E_CUDA;
    *ms_out = ms;
    return 0;
}

extern "C" int32_t ctsmg_measure_fp64_lane_cost(int32_t active_lanes, float* ms_out) {
    if (!ms_out || active_lanes < 1 || active_lanes > 32) return CTSMG_E_ARG;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return CTSMG_E_CUDA;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return CTSMG_E_CUDA;
    double* d = nullptr;
    if (cudaMalloc(&d, 8) != cudaSuccess) return CTSMG_E_CUDA;
    const int threads = 256, blocks = nsm * 8, iters = 512;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    dfma_loop_lanes<<<blocks, threads>>>(d, 16, 0.999999, 1e-7, active_lanes);
    cudaEventRecord(e0);
    dfma_loop_lanes<<<blocks, threads>>>(d, iters, 0.999999, 1e-7, active_lanes);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    if (err != cudaSuccess || ms <= 0.f) return CTSMG_E_CUDA;
    *ms_out = ms;
    return 0;
}

extern "C" int32_t ctsmg_measure_fp64_tflops(double* tflops) {
    if (!tflops) return CTSMG_E_ARG;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return CTSMG_E_CUDA;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return CTSMG_E_CUDA;
    double* d = nullptr;
    if (cudaMalloc(&d, 8) != cudaSuccess) return CTSMG_E_CUDA;
    const int threads = 256, blocks = nsm * 8, iters = 2048;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    dfma_loop<<<blocks, threads>>>(d, 64, 0.999999, 1e-7);     // warm-up
    cudaEventRecord(e0);
    dfma_loop<<<blocks, threads>>>(d, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    if (err != cudaSuccess || ms <= 0.f) return CTSMG_E_CUDA;
    const double flops = 2.0 * 8 * 16 * (double)iters * threads * blocks;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return 0;
}
