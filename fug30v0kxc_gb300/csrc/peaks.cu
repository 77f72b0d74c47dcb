// peaks.cu -- measured FP64 throughput of the GPU, the roofline denominator
// of the plain FP64 form (whose kernels are bound by the FP64 pipe, not by
// HBM).  No reference counterpart: instrumentation.
//
// Every thread runs CHAINS independent fused multiply-add chains for a fixed
// number of iterations; the grid fills every SM several times over, so the
// FP64 pipe, not the dependency latency, limits the rate.  The chains' final
// values are summed into one store per thread so that no FMA is dead code.
#include <stdio.h>

#include "common.cuh"

#define PEAK_CHAINS 8

__global__ void __launch_bounds__(256) k_dfma_peak(double *out, int iters, double b, double c)
{
    double a[PEAK_CHAINS];
#pragma unroll
    for (int q = 0; q < PEAK_CHAINS; q++) a[q] = (double)(threadIdx.x + q) * 1e-9;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int q = 0; q < PEAK_CHAINS; q++) a[q] = fma(a[q], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < PEAK_CHAINS; q++) s += a[q];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// FP64 FMA throughput of the current device in TFLOP/s (2 flops per FMA),
// the best of `reps` timed launches after one warm-up launch
extern "C" int vec_measure_fp64(int reps, double *tflops)
{
    if (!tflops || reps < 1) return VEC_ERR_ARG;
    int dev = 0, sms = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, threads = 256, iters = 4096;
    double *out = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int st = VEC_OK;
    float best = 1e30f;
    if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        cudaGetLastError();
        vec_set_error("vec_measure_fp64: set-up failed");
        st = VEC_ERR_CUDA;
    }
    for (int r = -1; r < reps && st == VEC_OK; r++) {
        cudaEventRecord(e0, s);
        k_dfma_peak<<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-7);
        cudaEventRecord(e1, s);
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
            vec_set_error("vec_measure_fp64: kernel failed");
            st = VEC_ERR_CUDA;
            break;
        }
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r >= 0 && ms < best) best = ms;
    }
    if (st == VEC_OK)
        *tflops = 2.0 * PEAK_CHAINS * (double)iters * blocks * threads / (best * 1e-3) / 1e12;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    if (out) cudaFree(out);
    return st;
}
