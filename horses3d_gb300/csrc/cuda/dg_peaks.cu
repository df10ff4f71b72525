// Measurement helper: the FP64 fused multiply-add rate of the current device, the denominator of the
// plain (all-FP64) form's compute roofline. Not a reference routine.
//
// Every thread runs kChains independent FMA chains (a = a*b + c) for `iters` rounds, enough
// independent work per warp to keep the FP64 pipe issuing every cycle; the grid fills every SM
// several times over. Timed with CUDA events on a private stream after one warm-up launch.
#include <cuda_runtime.h>

#include <string>

#include "../host/status.hpp"
#include "horses3d_gb300.h"

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_fp64_fma(double* out, int iters, double b, double c) {
    double a[kChains];
#pragma unroll
    for (int q = 0; q < kChains; ++q) a[q] = 1.0 + 1e-3 * (threadIdx.x + q);
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int q = 0; q < kChains; ++q) a[q] = fma(a[q], b, c);
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < kChains; ++q) s += a[q];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

}  // namespace

extern "C" int dg_measure_fp64_peak(double* tflops) {
    if (!tflops) return h3d::fail(DG_ERR_INVALID, "null argument");
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return h3d::fail(DG_ERR_NODEVICE, std::string("dg_measure_fp64_peak: ") + cudaGetErrorString(e));
    const int blocks = sms * 8;
    const int iters = 4096;
    double* out = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    float ms = 0.0f;
    e = cudaMalloc(&out, sizeof(double) * blocks * kThreads);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&t0);
    if (e == cudaSuccess) e = cudaEventCreate(&t1);
    if (e == cudaSuccess) {
        // b slightly below 1 and c small keep the values finite and normal for every round
        k_fp64_fma<<<blocks, kThreads, 0, s>>>(out, iters, 0.999999, 1e-6);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(t0, s);
    if (e == cudaSuccess) {
        k_fp64_fma<<<blocks, kThreads, 0, s>>>(out, iters, 0.999999, 1e-6);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(t1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(t1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    if (s) cudaStreamDestroy(s);
    if (out) cudaFree(out);
    if (e != cudaSuccess) return h3d::fail(DG_ERR_CUDA, std::string("dg_measure_fp64_peak: ") + cudaGetErrorString(e));
    const double flop = 2.0 * kChains * static_cast<double>(iters) * blocks * kThreads;
    *tflops = flop / (ms * 1e-3) / 1e12;
    return DG_OK;
}
