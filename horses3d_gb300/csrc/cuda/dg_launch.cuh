// Launch wrappers: one RK stage (five kernels) for a given (P, node family, arithmetic type), plus
// the order-independent reduction kernels (CFL time step, residuals) and the time advance.
#pragma once
#include <cuda_runtime.h>

#include "dg_kernels.cuh"

namespace dg {

// One stage of the RHS. stage -1: RHS only; 0..2: RHS + RK3 stage update (+ traces of the new
// state); kTraces: Q traces of the current state only; kPrepare: set kernel attributes, no launch.
// flags: kStoreGrad writes the lifted gradient, kWriteQDot stores the final QDot.
constexpr int kPrepare = -2;
constexpr int kTraces = -3;
constexpr int kStoreGrad = 1;
constexpr int kWriteQDot = 2;

template <typename R>
using StageFn = cudaError_t (*)(const Args<R>& a, int stage, double tshift, int flags, cudaStream_t s);

template <int P, typename R>
size_t volume_smem_bytes(int inviscid) {
    return static_cast<size_t>(Geo<P>::EPB) * volume_smem_values<P>(inviscid != 0) * sizeof(R);
}

template <int P, bool GL, typename R>
cudaError_t run_stage(const Args<R>& a, int stage, double tshift, int flags, cudaStream_t s) {
    constexpr int EPB = Geo<P>::EPB, THREADS = Geo<P>::THREADS;
    const int eblocks = (a.K + EPB - 1) / EPB;
    const long long fp = static_cast<long long>(a.F) * P * P;
    const int fblocks = static_cast<int>((fp + 127) / 128);
    if (stage == kPrepare)  // opt in to the large dynamic shared memory once, outside any capture
        return cudaFuncSetAttribute(k_volume<P, GL, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(volume_smem_bytes<P, R>(1)));
    if (stage == kTraces) {
        k_traces<P, GL, R><<<eblocks, THREADS, 0, s>>>(a);
        return cudaGetLastError();
    }
    k_volume<P, GL, R><<<eblocks, THREADS, volume_smem_bytes<P, R>(a.inviscid), s>>>(a, flags & kStoreGrad);
    k_flux<P, R><<<fblocks, 128, 0, s>>>(a);
    if (a.source) k_update<P, GL, true, R><<<eblocks, THREADS, 0, s>>>(a, stage, tshift, (flags & kWriteQDot) ? 1 : 0);
    else k_update<P, GL, false, R><<<eblocks, THREADS, 0, s>>>(a, stage, tshift, (flags & kWriteQDot) ? 1 : 0);
    return cudaGetLastError();
}

// Average device time of each kernel alone, measured with CUDA events on stream s over reps
// launches (k_update runs its RK stage-1 update). ms[0..3]: volume, flux, update, traces.
template <typename R>
using KernelTimesFn = cudaError_t (*)(const Args<R>& a, int reps, cudaStream_t s, double* ms);

template <int P, bool GL, typename R>
cudaError_t kernel_times(const Args<R>& a, int reps, cudaStream_t s, double* ms) {
    constexpr int EPB = Geo<P>::EPB, THREADS = Geo<P>::THREADS;
    const int eblocks = (a.K + EPB - 1) / EPB;
    const long long fp = static_cast<long long>(a.F) * P * P;
    const int fblocks = static_cast<int>((fp + 127) / 128);
    cudaEvent_t e0, e1;
    cudaError_t err = cudaEventCreate(&e0);
    if (err != cudaSuccess) return err;
    if ((err = cudaEventCreate(&e1)) != cudaSuccess) {
        cudaEventDestroy(e0);
        return err;
    }
    for (int kk = 0; kk < 4; ++kk) {
        cudaEventRecord(e0, s);
        for (int r = 0; r < reps; ++r) {
            switch (kk) {
                case 0: k_volume<P, GL, R><<<eblocks, THREADS, volume_smem_bytes<P, R>(a.inviscid), s>>>(a, 0); break;
                case 1: k_flux<P, R><<<fblocks, 128, 0, s>>>(a); break;
                case 2: k_update<P, GL, false, R><<<eblocks, THREADS, 0, s>>>(a, 1, 1.0 / 3.0, 0); break;
                default: k_traces<P, GL, R><<<eblocks, THREADS, 0, s>>>(a); break;
            }
        }
        cudaEventRecord(e1, s);
        if ((err = cudaEventSynchronize(e1)) != cudaSuccess) break;
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        ms[kk] = reps > 0 ? t / reps : 0.0;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err != cudaSuccess) return err;
    return cudaGetLastError();
}

// Resolved in the instantiation translation units.
StageFn<double> stage_fn_fp64(int P, bool gl);
StageFn<float> stage_fn_fp32(int P, bool gl);
KernelTimesFn<double> times_fn_fp64(int P, bool gl);
KernelTimesFn<float> times_fn_fp32(int P, bool gl);

// ------------------------------------------------------------------------ reductions ----------
// Non-negative doubles order like their bit patterns, so atomicMin/atomicMax on the 64-bit image
// implement min/max reductions exactly.
__device__ __forceinline__ unsigned long long dbits(double x) { return static_cast<unsigned long long>(__double_as_longlong(x)); }

struct DtArgs {
    long long ndof;
    double cfl, dcfl, dxi[3], dxi2[3];
    int ns;
    double gamma, gm1, gammaM2, S_div_TRef, TReNorm;
    const double* Q;
    unsigned long long* red;  // [0] convective, [1] viscous (bit images)
};

// MaxTimeStep (DGSEMClass.f90:870-1038) per node, block-reduced, then atomically folded.
template <typename R>
__global__ void k_max_dt(DtArgs d, const R* ja_xi, const R* ja_eta, const R* ja_zeta, const R* jac) {
    double conv = 1.0e300, visc = 1.0e300;
    for (long long g = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; g < d.ndof;
         g += static_cast<long long>(gridDim.x) * blockDim.x) {
        const double* Q = d.Q + 5 * g;
        const double p = d.gm1 * (Q[4] - 0.5 * (Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]) / Q[0]);
        const double a = sqrt(d.gamma * p / Q[0]);
        const double ev[3] = {fabs(Q[1] / Q[0]) + a, fabs(Q[2] / Q[0]) + a, fabs(Q[3] / Q[0]) + a};
        const R* ja[3] = {ja_xi + 3 * g, ja_eta + 3 * g, ja_zeta + 3 * g};
        double lam = 0.0, lamv = 0.0;
        const double J = fabs(double(jac[g]));
        double l3[3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
            l3[r] = fabs(double(ja[r][0]) * ev[0] + double(ja[r][1]) * ev[1] + double(ja[r][2]) * ev[2]) * d.dxi[r];
        lam = l3[0] + l3[1] + l3[2];
        conv = fmin(conv, d.cfl * J / lam);
        if (d.ns) {
            const double T = d.gammaM2 * p / Q[0];
            const double t = T * d.TReNorm;
            const double mu = (1.0 + d.S_div_TRef) / (t + d.S_div_TRef) * t * sqrt(t);
            double v3[3];
#pragma unroll
            for (int r = 0; r < 3; ++r)
                v3[r] = mu * d.dxi2[r] * fabs(double(ja[r][0]) + double(ja[r][1]) + double(ja[r][2]));
            lamv = v3[0] + v3[1] + v3[2];
            visc = fmin(visc, d.dcfl * J / lamv);
        }
    }
    __shared__ double sc[32], sv[32];
    for (int o = 16; o > 0; o >>= 1) {
        conv = fmin(conv, __shfl_down_sync(0xffffffffu, conv, o));
        visc = fmin(visc, __shfl_down_sync(0xffffffffu, visc, o));
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { sc[w] = conv; sv[w] = visc; }
    __syncthreads();
    if (w == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        conv = lane < nw ? sc[lane] : 1.0e300;
        visc = lane < nw ? sv[lane] : 1.0e300;
        for (int o = 16; o > 0; o >>= 1) {
            conv = fmin(conv, __shfl_down_sync(0xffffffffu, conv, o));
            visc = fmin(visc, __shfl_down_sync(0xffffffffu, visc, o));
        }
        if (lane == 0) {
            atomicMin(&d.red[0], dbits(conv));
            atomicMin(&d.red[1], dbits(visc));
        }
    }
}

// dt = min(convective, viscous); resets the reduction slots for the next use.
static __global__ void k_dt_final(unsigned long long* red, double* dt) {
    const double conv = __longlong_as_double(static_cast<long long>(red[0]));
    const double visc = __longlong_as_double(static_cast<long long>(red[1]));
    *dt = conv < visc ? conv : visc;
    red[0] = dbits(1.0e300);
    red[1] = dbits(1.0e300);
}

static __global__ void k_advance_time(double* t, const double* dt) { *t = *t + *dt; }

// ComputeMaxResiduals (DGSEMClass.f90:770-868) and the NaN test of checkForNan.
template <typename R>
__global__ void k_residuals(long long ndof, const R* qdot, const double* Q, unsigned long long* red, int* nan_flag) {
    double m[5] = {0, 0, 0, 0, 0};
    int bad = 0;
    for (long long g = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; g < ndof;
         g += static_cast<long long>(gridDim.x) * blockDim.x) {
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            m[v] = fmax(m[v], fabs(double(qdot[5 * g + v])));
            const double q = Q[5 * g + v];
            if (!(q == q) || fabs(q) > 1.7976931348623157e308) bad = 1;
        }
    }
#pragma unroll
    for (int v = 0; v < 5; ++v)
        for (int o = 16; o > 0; o >>= 1) m[v] = fmax(m[v], __shfl_down_sync(0xffffffffu, m[v], o));
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int v = 0; v < 5; ++v) atomicMax(&red[v], dbits(m[v]));
    }
    if (bad) atomicOr(nan_flag, 1);
}

}  // namespace dg
