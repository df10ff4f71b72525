// Self-test of the tensor-core building blocks (dg_tc.cuh): one CTA computes C = A B^T for
// A 128 x 8 and B 16 x 8 (FP32 inputs, row-major) with tcgen05 TF32 MMAs accumulated in TMEM, either
// as one TF32 product (split = 0) or as the three-term TF32 split product (split = 1), and reads C
// back through tcgen05.ld. It pins the operand layout, the descriptors and the TMEM access pattern
// that the tensor-core volume kernel uses. No reference counterpart.
#include <cuda_runtime.h>

#include <string>

#include "../host/status.hpp"
#include "dg_tc.cuh"
#include "horses3d_gb300.h"

namespace {

constexpr int kM = 128, kN = 16, kK = 8;

__global__ void __launch_bounds__(128) k_tc_selftest(const float* __restrict__ A, const float* __restrict__ B,
                                                     float* __restrict__ Cout, int split, int* err) {
    using namespace dg;
    __shared__ __align__(1024) unsigned char sA[2][tc::operand_bytes(kM)];
    __shared__ __align__(1024) unsigned char sB[2][tc::operand_bytes(kN)];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tslot;
    const int t = threadIdx.x, warp = t >> 5;
    if (warp == 0) {
        tc::tmem_alloc(&tslot, 32);
        tc::fence_before_sync();
    }
    // operands: hi and lo parts in the canonical layout
    for (int k = 0; k < kK; ++k) {
        const float x = A[t * kK + k];
        const float hi = tc::tf32_hi(x);
        *reinterpret_cast<float*>(sA[0] + tc::operand_offset(t, k)) = hi;
        *reinterpret_cast<float*>(sA[1] + tc::operand_offset(t, k)) = x - hi;
        if (t < kN) {
            const float y = B[t * kK + k];
            const float yh = tc::tf32_hi(y);
            *reinterpret_cast<float*>(sB[0] + tc::operand_offset(t, k)) = yh;
            *reinterpret_cast<float*>(sB[1] + tc::operand_offset(t, k)) = y - yh;
        }
    }
    if (t == 0) {
        mbar_init(&bar, 1);
        mbar_init_fence();
    }
    fence_proxy_async_smem();  // the operand stores before the tensor core reads them
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t taddr = tslot;
    if (t == 0) {
        const uint32_t id = tc::idesc_tf32(kM, kN);
        tc::mma_tf32(taddr, tc::smem_desc(sA[0]), tc::smem_desc(sB[0]), id, false);
        if (split) {
            tc::mma_tf32(taddr, tc::smem_desc(sA[0]), tc::smem_desc(sB[1]), id, true);
            tc::mma_tf32(taddr, tc::smem_desc(sA[1]), tc::smem_desc(sB[0]), id, true);
        }
        tc::commit(&bar);
    }
    const bool done = mbar_wait(&bar, 0);
    const bool ok = !__syncthreads_or(!done);
    tc::fence_after_sync();
    if (ok) {
        float v[16];
        tc::ld_32x32b_x16(taddr + (static_cast<uint32_t>(32 * warp) << 16), v);
#pragma unroll
        for (int q = 0; q < kN; ++q) Cout[t * kN + q] = v[q];
    } else if (t == 0) {
        atomicOr(err, 1);
        mbar_wait(&bar, 0, kWaitNs / 4);  // bounded: let a late MMA finish before the TMEM is freed
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(taddr, 32);
}

}  // namespace

extern "C" int dg_tc_selftest(const float* a, const float* b, float* c, int split) {
    if (!a || !b || !c) return h3d::fail(DG_ERR_INVALID, "null argument");
    float *dA = nullptr, *dB = nullptr, *dC = nullptr;
    int* dErr = nullptr;
    int herr = 0;
    cudaError_t e = cudaMalloc(&dA, sizeof(float) * kM * kK);
    if (e == cudaSuccess) e = cudaMalloc(&dB, sizeof(float) * kN * kK);
    if (e == cudaSuccess) e = cudaMalloc(&dC, sizeof(float) * kM * kN);
    if (e == cudaSuccess) e = cudaMalloc(&dErr, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(dErr, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(dA, a, sizeof(float) * kM * kK, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dB, b, sizeof(float) * kN * kK, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_tc_selftest<<<1, 128>>>(dA, dB, dC, split, dErr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(c, dC, sizeof(float) * kM * kN, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&herr, dErr, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dC);
    cudaFree(dErr);
    if (e != cudaSuccess) return h3d::fail(DG_ERR_CUDA, std::string("dg_tc_selftest: ") + cudaGetErrorString(e));
    if (herr) return h3d::fail(DG_ERR_TIMEOUT, "dg_tc_selftest: the MMA completion wait gave up");
    return DG_OK;
}
