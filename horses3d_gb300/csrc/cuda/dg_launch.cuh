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
// The monitored device time loop: kFuseMonitor, the update of this stage writes the elements'
// residual records (a.mon words 0..5); kEstimateDt, the volume kernel of this stage writes the
// elements' time-step estimates (words 6, 7).
constexpr int kFuseMonitor = 16;
constexpr int kEstimateDt = 32;

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

// The monitored time loop's estimate variant of the volume kernel exists for the orders whose
// update stages element blocks by TMA (one element per CTA), as the fused residual records do.
template <int P>
constexpr bool kEstVolume = (P == 6);

template <int P, bool GL, typename R>
void launch_volume(const Args<R>& a, int blocks, int store_grad, cudaStream_t s, bool est = false) {
    if constexpr (kEstVolume<P>) {
        if (est) {
            k_volume<P, GL, R, false, true><<<blocks, Geo<P>::THREADS, volume_smem_bytes<P, R>(a.inviscid), s>>>(
                a, store_grad);
            return;
        }
    }
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

// fuse: the monitored time loop's last stage also writes each element's residual/NaN record and
// MaxTimeStep estimate (kTmaUpdate orders only).
template <int P, bool GL, bool SRC, typename R>
void launch_update(const Args<R>& a, int blocks, int stage, double tshift, int wq, cudaStream_t s, bool fuse = false) {
    if constexpr (kTmaUpdate<P>) {
        if (fuse) k_update_tma<P, GL, SRC, R, true><<<blocks, Geo<P>::THREADS, 0, s>>>(a, stage, tshift, wq);
        else k_update_tma<P, GL, SRC, R><<<blocks, Geo<P>::THREADS, 0, s>>>(a, stage, tshift, wq);
    } else {
        k_update<P, GL, SRC, R><<<blocks, Geo<P>::THREADS, 0, s>>>(a, stage, tshift, wq);
    }
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
        if constexpr (kEstVolume<P>) {
            const cudaError_t e = cudaFuncSetAttribute(k_volume<P, GL, R, false, true>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       static_cast<int>(volume_smem_bytes<P, R>(1)));
            if (e != cudaSuccess) return e;
        }
        return cudaFuncSetAttribute(k_volume<P, GL, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    static_cast<int>(volume_smem_bytes<P, R>(1)));
    }
    if (stage == kTraces) {
        k_traces<P, GL, R><<<eblocks, THREADS, 0, s>>>(a);
        return cudaGetLastError();
    }
    if (!(flags & kSurfaceOnly)) launch_volume<P, GL, R>(a, eblocks, flags & kStoreGrad, s, (flags & kEstimateDt) != 0);
    if (flags & kVolumeOnly) return cudaGetLastError();
    launch_flux<P, R>(a, fblocks, s);
    const bool fuse = (flags & kFuseMonitor) != 0;
    if (a.source) launch_update<P, GL, true>(a, eblocks, stage, tshift, (flags & kWriteQDot) ? 1 : 0, s, fuse);
    else launch_update<P, GL, false>(a, eblocks, stage, tshift, (flags & kWriteQDot) ? 1 : 0, s, fuse);
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

// ------------------------------------------------------------------ fused time-loop monitor ----
// The monitored device time loop (dg_integrate) of the orders with the one-element-per-CTA volume and
// update kernels needs no separate pass over Q, QDot and the geometry for its monitor: per element
// a record of 8 words (a.mon) is filled by the kernels that hold the data anyway.
//   stage 1   k_volume<EST>: FP32 MaxTimeStep estimates of the step's initial state (words 6, 7);
//             k_estimate_fold -> red[7]; k_dt_exact_elem (elements whose estimate lies in the
//             window) + k_dt_final -> dt; then the stage's flux and update kernels
//   stage 3   k_update_tma<FUSE>: max |QDot| per variable and the NaN/Inf flag of the new state
//             (words 0..5); after the step k_monitor_fold -> red[2..6], the NaN flag, the history row
// The dt equals the two-pass reduction's bit for bit (the same window argument, per element instead
// of per chunk), and the residuals equal k_residuals' (maxima of the same values).
constexpr int kFoldBlocks = 152;

// Folds the element records' residual words into red[2..6] (max |QDot|) and *nan_flag.
__global__ static void __launch_bounds__(256) k_monitor_fold(const unsigned long long* __restrict__ mon, int K,
                                                             unsigned long long* red, int* nan_flag) {
    unsigned long long m[5] = {0, 0, 0, 0, 0};
    int b = 0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < K; e += gridDim.x * blockDim.x) {
        const unsigned long long* r = mon + 8 * static_cast<int64_t>(e);
#pragma unroll
        for (int v = 0; v < 5; ++v) m[v] = r[v] > m[v] ? r[v] : m[v];
        b |= r[5] != 0;
    }
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            const unsigned long long x = __shfl_down_sync(0xffffffffu, m[v], o);
            m[v] = x > m[v] ? x : m[v];
        }
        b |= __shfl_down_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int v = 0; v < 5; ++v) atomicMax(&red[2 + v], m[v]);
        if (b) atomicOr(nan_flag, 1);
    }
}

// Folds the element records' estimate words into the FP32 minima of red[7] (which holds two FP32
// +inf on entry: k_dt_final leaves it so).
__global__ static void __launch_bounds__(256) k_estimate_fold(const unsigned long long* __restrict__ mon, int K,
                                                              unsigned long long* red) {
    unsigned c = 0xffffffffu, w = 0xffffffffu;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < K; e += gridDim.x * blockDim.x) {
        const unsigned long long* r = mon + 8 * static_cast<int64_t>(e);
        const unsigned rc = static_cast<unsigned>(r[6]), rw = static_cast<unsigned>(r[7]);
        c = rc < c ? rc : c;
        w = rw < w ? rw : w;
    }
    c = __reduce_min_sync(0xffffffffu, c);
    w = __reduce_min_sync(0xffffffffu, w);
    if ((threadIdx.x & 31) == 0) {
        unsigned int* s32 = reinterpret_cast<unsigned int*>(red + 7);
        atomicMin(&s32[0], c);
        atomicMin(&s32[1], w);
    }
}

// The exact pass: a grid of kExactBlocks CTAs strides over the elements; an element none of whose
// nodes can be in the window is skipped (a block-uniform test on its record).
constexpr int kExactBlocks = 4 * 152;
template <int P, typename R>
__global__ void __launch_bounds__(Geo<P>::THREADS) k_dt_exact_elem(Args<R> a, DtArgs d) {
    constexpr int NT = Geo<P>::P3;
    const int n = threadIdx.x;
    const unsigned int* s32 = reinterpret_cast<const unsigned int*>(d.red + 7);
    const float thr_c = __uint_as_float(s32[0]) * (1.0f + kDtWindow);
    const float thr_v = __uint_as_float(s32[1]) * (1.0f + kDtWindow);
    __shared__ double sc[NT], sv[NT];
    for (int e = blockIdx.x; e < a.K; e += gridDim.x) {
        const unsigned long long* rec = a.mon + 8 * static_cast<int64_t>(e);
        const float ec = __uint_as_float(static_cast<unsigned>(rec[6]));
        const float evs = __uint_as_float(static_cast<unsigned>(rec[7]));
        if (ec > thr_c && !(d.ns && !(evs > thr_v))) continue;  // block-uniform
        const int64_t g = static_cast<int64_t>(e) * NT + n;
        const double* Q = d.Q + 5 * g;
        float cv, vs;
        dt_estimate(a.dtc, Q, a.ja_xi + 3 * g, a.ja_eta + 3 * g, a.ja_zeta + 3 * g, a.jac[g], cv, vs);
        double conv = 1.0e300, visc = 1.0e300;
        const bool wc = !(cv > thr_c), wv = d.ns && !(vs > thr_v);
        if (wc || wv)
            dt_exact(d, d.dxi, d.dxi2, Q, a.ja_xi + 3 * g, a.ja_eta + 3 * g, a.ja_zeta + 3 * g, a.jac[g], d.gammaM2, wc,
                     wv, conv, visc);
        sc[n] = conv;
        sv[n] = visc;
        __syncthreads();
        if (n < 32) {
            for (int q = n + 32; q < NT; q += 32) {
                conv = fmin(conv, sc[q]);
                visc = fmin(visc, sv[q]);
            }
            for (int o = 16; o > 0; o >>= 1) {
                conv = fmin(conv, __shfl_down_sync(0xffffffffu, conv, o));
                visc = fmin(visc, __shfl_down_sync(0xffffffffu, visc, o));
            }
            if (n == 0) {
                atomicMin(&d.red[0], dbits(conv));
                atomicMin(&d.red[1], dbits(visc));
            }
        }
        __syncthreads();  // sc, sv are reused by the next element
    }
}

// MaxTimeStep from the estimate records of the current state: the estimate minima into red[7], the
// exact pass into red[0], red[1] (k_dt_final follows).
template <typename R>
struct MonitorFns {
    cudaError_t (*dt)(const Args<R>& a, const DtArgs& d, cudaStream_t s);
};

template <int P, bool GL, typename R>
cudaError_t monitor_dt(const Args<R>& a, const DtArgs& d, cudaStream_t s) {
    k_estimate_fold<<<kFoldBlocks, 256, 0, s>>>(a.mon, a.K, d.red);
    k_dt_exact_elem<P, R><<<a.K < kExactBlocks ? a.K : kExactBlocks, Geo<P>::THREADS, 0, s>>>(a, d);
    return cudaGetLastError();
}

// Resolved in the instantiation translation units.
MonitorFns<double> monitor_fns_fp64(int P, bool gl);
MonitorFns<float> monitor_fns_fp32(int P, bool gl);
StageFn<double> stage_fn_fp64(int P, bool gl);
StageFn<float> stage_fn_fp32(int P, bool gl);
KernelTimesFn<double> times_fn_fp64(int P, bool gl);
KernelTimesFn<float> times_fn_fp32(int P, bool gl);

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
