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
// Element partitions run a stage in two halves with halo exchanges before each: kVolumeOnly launches
// the volume kernel alone (after the ghost slots received the neighbours' Q traces), kSurfaceOnly the
// face flux and update kernels (after they received the neighbours' viscous normal fluxes).
constexpr int kVolumeOnly = 4;
constexpr int kSurfaceOnly = 8;

template <typename R>
using StageFn = cudaError_t (*)(const Args<R>& a, int stage, double tshift, int flags, cudaStream_t s);

template <int P, typename R>
size_t volume_smem_bytes(int inviscid) {
    return static_cast<size_t>(Geo<P>::EPB) * volume_smem_values<P, R>(inviscid != 0) * sizeof(R);
}

// The tensor-core gradient variant exists for the headline configuration: N = 5 on Gauss nodes,
// FP32 arithmetic (the mixed form), standard volume form.
template <int P, bool GL, typename R>
constexpr bool kTcVolume = (P == 6 && !GL && sizeof(R) == 4);

template <int P, typename R>
size_t volume_tc_smem_bytes() {
    return volume_tc_offset<P, R>() + TcLayout::BYTES;
}

template <int P, bool GL, typename R>
void launch_volume(const Args<R>& a, int blocks, int store_grad, cudaStream_t s) {
    if constexpr (kTcVolume<P, GL, R>) {
        if (a.tc) {
            k_volume<P, GL, R, true><<<blocks, Geo<P>::THREADS, volume_tc_smem_bytes<P, R>(), s>>>(a, store_grad);
            return;
        }
    }
    k_volume<P, GL, R><<<blocks, Geo<P>::THREADS, volume_smem_bytes<P, R>(a.inviscid), s>>>(a, store_grad);
}

// The update kernel stages its element blocks by TMA where one element fills the CTA and its
// FP64 blocks fit the static shared memory (P = 6, the headline order).
template <int P>
constexpr bool kTmaUpdate = (P == 6);

template <int P, bool GL, bool SRC, typename R>
void launch_update(const Args<R>& a, int blocks, int stage, double tshift, int wq, cudaStream_t s) {
    if constexpr (kTmaUpdate<P>) k_update_tma<P, GL, SRC, R><<<blocks, Geo<P>::THREADS, 0, s>>>(a, stage, tshift, wq);
    else k_update<P, GL, SRC, R><<<blocks, Geo<P>::THREADS, 0, s>>>(a, stage, tshift, wq);
}

// The interface-flux kernel in its common variant (Roe, LxF, central, Rusanov, u-diss with the
// averages 0-4) or the generic one with the other solvers and the logarithmic-mean averages.
template <int P, typename R>
void launch_flux(const Args<R>& a, int blocks, cudaStream_t s) {
    if ((a.ph.riemann >= 4 && a.ph.riemann <= 8) || a.ph.averaging >= 5) k_flux<P, R, true><<<blocks, 128, 0, s>>>(a);
    else k_flux<P, R, false><<<blocks, 128, 0, s>>>(a);
}

template <int P, bool GL, typename R>
cudaError_t run_stage(const Args<R>& a, int stage, double tshift, int flags, cudaStream_t s) {
    constexpr int EPB = Geo<P>::EPB, THREADS = Geo<P>::THREADS;
    const int eblocks = (a.K + EPB - 1) / EPB;
    const long long fp = static_cast<long long>(a.F) * P * P;
    const int fblocks = static_cast<int>((fp + 127) / 128);
    if (stage == kPrepare) {  // opt in to the large dynamic shared memory once, outside any capture
        if constexpr (kTcVolume<P, GL, R>) {
            const cudaError_t e = cudaFuncSetAttribute(k_volume<P, GL, R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       static_cast<int>(volume_tc_smem_bytes<P, R>()));
            if (e != cudaSuccess) return e;
        }
        return cudaFuncSetAttribute(k_volume<P, GL, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(volume_smem_bytes<P, R>(1)));
    }
    if (stage == kTraces) {
        k_traces<P, GL, R><<<eblocks, THREADS, 0, s>>>(a);
        return cudaGetLastError();
    }
    if (!(flags & kSurfaceOnly)) launch_volume<P, GL, R>(a, eblocks, flags & kStoreGrad, s);
    if (flags & kVolumeOnly) return cudaGetLastError();
    launch_flux<P, R>(a, fblocks, s);
    if (a.source) launch_update<P, GL, true>(a, eblocks, stage, tshift, (flags & kWriteQDot) ? 1 : 0, s);
    else launch_update<P, GL, false>(a, eblocks, stage, tshift, (flags & kWriteQDot) ? 1 : 0, s);
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
                case 0: launch_volume<P, GL, R>(a, eblocks, 0, s); break;
                case 1: launch_flux<P, R>(a, fblocks, s); break;
                case 2: launch_update<P, GL, false>(a, eblocks, 1, 1.0 / 3.0, 0, s); break;
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

// |x| as its bit pattern (float: 31 bits, double: 63 bits); the maximum of such patterns is the
// pattern of the maximum |x|.
__device__ __forceinline__ unsigned long long abs_bits(float x) { return __float_as_uint(x) & 0x7fffffffu; }
__device__ __forceinline__ unsigned long long abs_bits(double x) { return dbits(x) & 0x7fffffffffffffffull; }
// The double image (for the FP64 reduction slots) of a maximum pattern of the element type.
__device__ __forceinline__ unsigned long long abs_bits_as_double(unsigned long long m, const float*) {
    return dbits(static_cast<double>(__uint_as_float(static_cast<unsigned>(m))));
}
__device__ __forceinline__ unsigned long long abs_bits_as_double(unsigned long long m, const double*) { return m; }
// NaN or Inf: all exponent bits set.
__device__ __forceinline__ int nonfinite(double x) { return (dbits(x) & 0x7ff0000000000000ull) == 0x7ff0000000000000ull; }

struct DtArgs {
    long long ndof;
    double cfl, dcfl, dxi[3], dxi2[3];
    int ns;
    double gamma, gm1, gammaM2, S_div_TRef, TReNorm;
    const double* Q;
    unsigned long long* red;  // [0] convective, [1] viscous (FP64 bit images), [7] FP32 estimates (2 x 32 bit)
};

// MaxTimeStep (DGSEMClass.f90:870-1038) in two passes. The minimum is taken over FP64 quotients
// that need about ten FP64 divisions and square roots per node, so evaluating every node in FP64
// costs milliseconds on a part whose FP64 rate is 1/64 of FP32. Pass 1 estimates each node's
// convective and viscous limits in FP32 and reduces their minima m32. Pass 2 repeats the estimate
// and evaluates the exact FP64 expressions only at nodes whose estimate is within kDtWindow of m32
// (or not a number). An FP32 estimate differs from the FP64 value by a relative 1e-6 or less for
// physical states, far inside the window, so the node that attains the FP64 minimum is always
// evaluated and the result equals the FP64 minimum over all nodes bit for bit.
constexpr float kDtWindow = 1.0e-3f;
constexpr unsigned long long kDtEstimateInit = 0x7F8000007F800000ull;  // two FP32 +inf

struct DtConst32 {
    float cfl, dcfl, dxi[3], dxi2[3], gamma, gm1, gammaM2, S_div_TRef, TReNorm;
    int ns;
};

__host__ __device__ inline DtConst32 dt_const32(double cfl, double dcfl, const double* dxi, double gamma, double gm1,
                                                double gammaM2, double S_div_TRef, double TReNorm, int ns) {
    DtConst32 c;
    c.cfl = float(cfl);
    c.dcfl = float(dcfl);
    for (int r = 0; r < 3; ++r) {
        c.dxi[r] = float(dxi[r]);
        c.dxi2[r] = float(dxi[r] * dxi[r]);
    }
    c.gamma = float(gamma);
    c.gm1 = float(gm1);
    c.gammaM2 = float(gammaM2);
    c.S_div_TRef = float(S_div_TRef);
    c.TReNorm = float(TReNorm);
    c.ns = ns;
    return c;
}

// FP32 estimates of one node's convective and viscous time-step limits.
template <typename R>
__device__ __forceinline__ void dt_estimate(const DtConst32& d, const double* Q, const R* jx, const R* je, const R* jz,
                                            R jac, float& conv, float& visc) {
    const float rho = to_f32(Q[0]), ru = to_f32(Q[1]), rv = to_f32(Q[2]), rw = to_f32(Q[3]), E = to_f32(Q[4]);
    const float ir = 1.0f / rho;
    const float p = d.gm1 * (E - 0.5f * (ru * ru + rv * rv + rw * rw) * ir);
    const float a = sqrtf(d.gamma * p * ir);
    const float ev[3] = {fabsf(ru * ir) + a, fabsf(rv * ir) + a, fabsf(rw * ir) + a};
    const float J = fabsf(float(jac));
    const R* ja[3] = {jx, je, jz};
    float lam = 0.0f;
#pragma unroll
    for (int r = 0; r < 3; ++r)
        lam += fabsf(float(ja[r][0]) * ev[0] + float(ja[r][1]) * ev[1] + float(ja[r][2]) * ev[2]) * d.dxi[r];
    conv = d.cfl * J / lam;
    visc = 3.0e38f;
    if (d.ns) {
        const float t = d.gammaM2 * p * ir * d.TReNorm;
        const float mu = (1.0f + d.S_div_TRef) / (t + d.S_div_TRef) * t * sqrtf(t);
        float lv = 0.0f;
#pragma unroll
        for (int r = 0; r < 3; ++r) lv += mu * d.dxi2[r] * fabsf(float(ja[r][0]) + float(ja[r][1]) + float(ja[r][2]));
        visc = d.dcfl * J / lv;
    }
}

// The exact FP64 limits of one node (the reference's expressions and operation order).
template <typename R>
__device__ __forceinline__ void dt_exact(const DtArgs& d, const double* dx, const double* dx2, const double* Q,
                                         const R* jx, const R* je, const R* jz, R jac, double gammaM2, bool want_conv,
                                         bool want_visc, double& conv, double& visc) {
    const double p = d.gm1 * (Q[4] - 0.5 * (Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]) / Q[0]);
    const double J = fabs(double(jac));
    const R* ja[3] = {jx, je, jz};
    if (want_conv) {
        const double a = sqrt(d.gamma * p / Q[0]);
        const double ev[3] = {fabs(Q[1] / Q[0]) + a, fabs(Q[2] / Q[0]) + a, fabs(Q[3] / Q[0]) + a};
        double l3[3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
            l3[r] = fabs(double(ja[r][0]) * ev[0] + double(ja[r][1]) * ev[1] + double(ja[r][2]) * ev[2]) * dx[r];
        conv = d.cfl * J / (l3[0] + l3[1] + l3[2]);
    }
    if (want_visc) {
        const double T = gammaM2 * p / Q[0];
        const double t = T * d.TReNorm;
        const double mu = (1.0 + d.S_div_TRef) / (t + d.S_div_TRef) * t * sqrt(t);
        double v3[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) v3[r] = mu * dx2[r] * fabs(double(ja[r][0]) + double(ja[r][1]) + double(ja[r][2]));
        visc = d.dcfl * J / (v3[0] + v3[1] + v3[2]);
    }
}

__device__ __forceinline__ unsigned int fbits(float x) { return __float_as_uint(x); }

// Block minimum of two values, folded into the 64-bit (double) or 32-bit (float) slots by atomicMin on
// the bit images (non-negative values order like their bit patterns).
template <typename T>
__device__ __forceinline__ void block_min2(T a, T b, T* slot_a_out, T* slot_b_out) {
    __shared__ T sa[32], sb[32];
    for (int o = 16; o > 0; o >>= 1) {
        a = fmin(a, __shfl_down_sync(0xffffffffu, a, o));
        b = fmin(b, __shfl_down_sync(0xffffffffu, b, o));
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        sa[w] = a;
        sb[w] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        for (int q = 1; q < nw; ++q) {
            a = fmin(a, sa[q]);
            b = fmin(b, sb[q]);
        }
        *slot_a_out = a;
        *slot_b_out = b;
    }
}

// Each block takes one contiguous chunk of nodes in both passes, and the estimate pass records the
// chunk's minima (bmin[2b], bmin[2b+1]), so that the exact pass skips every chunk without a node in
// the window of the global minimum.
__device__ __forceinline__ void dt_chunk(long long ndof, long long& g0, long long& g1) {
    const long long chunk = (ndof + gridDim.x - 1) / gridDim.x;
    g0 = blockIdx.x * chunk;
    g1 = g0 + chunk < ndof ? g0 + chunk : ndof;
}

template <typename R>
__global__ void k_dt_estimate(DtConst32 c, long long ndof, const double* Q, const R* ja_xi, const R* ja_eta,
                              const R* ja_zeta, const R* jac, unsigned long long* red, float* bmin) {
    float conv = 3.0e38f, visc = 3.0e38f;
    long long g0, g1;
    dt_chunk(ndof, g0, g1);
    for (long long g = g0 + threadIdx.x; g < g1; g += blockDim.x) {
        float cv, vs;
        dt_estimate(c, Q + 5 * g, ja_xi + 3 * g, ja_eta + 3 * g, ja_zeta + 3 * g, jac[g], cv, vs);
        conv = fminf(conv, cv);
        visc = fminf(visc, vs);
    }
    float bc, bv;
    block_min2(conv, visc, &bc, &bv);
    if (threadIdx.x == 0) {
        unsigned int* s32 = reinterpret_cast<unsigned int*>(red + 7);
        atomicMin(&s32[0], fbits(bc));
        atomicMin(&s32[1], fbits(bv));
        bmin[2 * blockIdx.x] = bc;
        bmin[2 * blockIdx.x + 1] = bv;
    }
}

template <typename R>
__global__ void k_dt_exact(DtArgs d, DtConst32 c, const R* ja_xi, const R* ja_eta, const R* ja_zeta, const R* jac,
                           const float* bmin) {
    const unsigned int* s32 = reinterpret_cast<const unsigned int*>(d.red + 7);
    const float thr_c = __uint_as_float(s32[0]) * (1.0f + kDtWindow);
    const float thr_v = __uint_as_float(s32[1]) * (1.0f + kDtWindow);
    // no node of this chunk is a candidate: nothing to add (a block-uniform exit, before any barrier)
    if (bmin[2 * blockIdx.x] > thr_c && !(d.ns && !(bmin[2 * blockIdx.x + 1] > thr_v))) return;
    double conv = 1.0e300, visc = 1.0e300;
    long long g0, g1;
    dt_chunk(d.ndof, g0, g1);
    for (long long g = g0 + threadIdx.x; g < g1; g += blockDim.x) {
        const double* Q = d.Q + 5 * g;
        float cv, vs;
        dt_estimate(c, Q, ja_xi + 3 * g, ja_eta + 3 * g, ja_zeta + 3 * g, jac[g], cv, vs);
        const bool wc = !(cv > thr_c), wv = d.ns && !(vs > thr_v);
        if (wc || wv) {
            double ec = 1.0e300, evv = 1.0e300;
            dt_exact(d, d.dxi, d.dxi2, Q, ja_xi + 3 * g, ja_eta + 3 * g, ja_zeta + 3 * g, jac[g], d.gammaM2, wc, wv, ec, evv);
            conv = fmin(conv, ec);
            visc = fmin(visc, evv);
        }
    }
    double bc, bv;
    block_min2(conv, visc, &bc, &bv);
    if (threadIdx.x == 0) {
        atomicMin(&d.red[0], dbits(bc));
        atomicMin(&d.red[1], dbits(bv));
    }
}

// dt = min(convective, viscous); resets the reduction slots for the next use.
static __global__ void k_dt_final(unsigned long long* red, double* dt) {
    const double conv = __longlong_as_double(static_cast<long long>(red[0]));
    const double visc = __longlong_as_double(static_cast<long long>(red[1]));
    *dt = conv < visc ? conv : visc;
    red[0] = dbits(1.0e300);
    red[1] = dbits(1.0e300);
    red[7] = kDtEstimateInit;
}

static __global__ void k_advance_time(double* t, const double* dt) { *t = *t + *dt; }

// ComputeMaxResiduals (DGSEMClass.f90:770-868) and the NaN test of checkForNan.
template <typename R>
__global__ void k_residuals(long long ndof, const R* qdot, const double* Q, unsigned long long* red, int* nan_flag) {
    // max |QDot| and the NaN/Inf test on bit patterns (non-negative IEEE numbers order as their bits),
    // so that the pass runs on the integer pipe instead of the slow FP64 one
    unsigned long long m[5] = {0, 0, 0, 0, 0};
    int bad = 0;
    for (long long g = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; g < ndof;
         g += static_cast<long long>(gridDim.x) * blockDim.x) {
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            const unsigned long long a = abs_bits(qdot[5 * g + v]);
            m[v] = a > m[v] ? a : m[v];
            bad |= nonfinite(Q[5 * g + v]);
        }
    }
#pragma unroll
    for (int v = 0; v < 5; ++v)
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long x = __shfl_down_sync(0xffffffffu, m[v], o);
            m[v] = x > m[v] ? x : m[v];
        }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int v = 0; v < 5; ++v) atomicMax(&red[v], abs_bits_as_double(m[v], qdot));
    }
    if (bad) atomicOr(nan_flag, 1);
}

// Deterministic FP64 sum of Q[5g+4] over g in [g0, g1): a fixed grid (kSumBlocks blocks, grid-stride,
// fixed-order tree per block) writes per-block partial sums, one block adds them in order. The mixed
// form's energy reference is this sum over the node count.
constexpr int kSumBlocks = 512;
constexpr int kDtBlocks = 2 * 152 * 4;  // MaxTimeStep passes: one contiguous chunk of nodes per block
__global__ static void __launch_bounds__(256) k_energy_partial(long long g0, long long g1, const double* Q,
                                                               double* partial) {
    __shared__ double sh[256];
    double acc = 0.0;
    for (long long g = g0 + blockIdx.x * 256LL + threadIdx.x; g < g1; g += kSumBlocks * 256LL) acc += Q[5 * g + 4];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}
__global__ static void __launch_bounds__(256) k_energy_final(const double* partial, double* out) {
    __shared__ double sh[256];
    double acc = 0.0;
    for (int b = threadIdx.x; b < kSumBlocks; b += 256) acc += partial[b];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

// One history row per step (dg_integrate): per case the five residuals (bit images in red at
// red_stride * k + 2) and the NaN flag, at row *count, then ++*count. One thread.
__global__ static void k_record_monitor(const unsigned long long* red, int red_stride, const int* nan_flag,
                                        int n_cases, double* rows, int* count, int capacity) {
    const int r = *count;
    if (r >= capacity) return;
    double* row = rows + static_cast<long long>(r) * 6 * n_cases;
    for (int k = 0; k < n_cases; ++k) {
        for (int v = 0; v < 5; ++v) row[6 * k + v] = __longlong_as_double(static_cast<long long>(red[red_stride * k + 2 + v]));
        row[6 * k + 5] = nan_flag[k] ? 1.0 : 0.0;
    }
    *count = r + 1;
}

}  // namespace dg
