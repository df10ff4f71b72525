// Allocation-free variant of the CFL time-step reduction (MaxTimeStep, DGSEMClass.f90:870-1038).
//
// Some callers cannot call cudaMalloc: a host code that hands all device memory out of its own
// pool (a Fortran/OpenACC or CUDA-Fortran host that allocated the solution arrays itself), code that
// runs after an allocation freeze, or a caller that must not grow the device footprint between
// steps. dg_max_dt_noalloc serves them: the caller passes device pointers to its state and metric
// terms, and the only scratch memory, the per-block partial minima of the reduction, lives in a
// file-scope device array of fixed size that every GPU loading this library keeps until exit.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../host/spectral.hpp"
#include "../host/status.hpp"
#include "horses3d_gb300.h"

namespace {

constexpr int kThreads = 256;
constexpr int kNodesPerThread = 32;
constexpr int kNodesPerBlock = kThreads * kNodesPerThread;  // 8192 nodes reduced by one block
constexpr int kMaxBlocks = 8192;                             // -> at most 67,108,864 nodes

// Per-block (convective, viscous) minima; 128 KiB. Shared by every call on the device.
static __device__ __align__(256) double g_partials[2 * kMaxBlocks];

struct DtConst {
    long long ndof;
    double cfl, dcfl, dxi[3], dxi2[3];
    int ns;
    double gamma, gm1, gammaM2, S_div_TRef, TReNorm;
};

// Pass 1: block b reduces nodes [b*kNodesPerBlock, (b+1)*kNodesPerBlock) into partials[2b], [2b+1].
__global__ void k_dt_partials(DtConst d, const double* __restrict__ Q, const double* __restrict__ ja_xi,
                              const double* __restrict__ ja_eta, const double* __restrict__ ja_zeta,
                              const double* __restrict__ jac, double* partials) {
    double conv = 1.0e300, visc = 1.0e300;
    const long long base = static_cast<long long>(blockIdx.x) * kNodesPerBlock;
    for (int r = 0; r < kNodesPerThread; ++r) {
        const long long g = base + static_cast<long long>(r) * kThreads + threadIdx.x;
        if (g >= d.ndof) break;
        const double* q = Q + 5 * g;
        const double p = d.gm1 * (q[4] - 0.5 * (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]) / q[0]);
        const double a = sqrt(d.gamma * p / q[0]);
        const double ev[3] = {fabs(q[1] / q[0]) + a, fabs(q[2] / q[0]) + a, fabs(q[3] / q[0]) + a};
        const double* ja[3] = {ja_xi + 3 * g, ja_eta + 3 * g, ja_zeta + 3 * g};
        const double J = fabs(jac[g]);
        double l3[3];
        for (int k = 0; k < 3; ++k) l3[k] = fabs(ja[k][0] * ev[0] + ja[k][1] * ev[1] + ja[k][2] * ev[2]) * d.dxi[k];
        conv = fmin(conv, d.cfl * J / (l3[0] + l3[1] + l3[2]));
        if (d.ns) {
            const double t = d.gammaM2 * p / q[0] * d.TReNorm;
            const double mu = (1.0 + d.S_div_TRef) / (t + d.S_div_TRef) * t * sqrt(t);
            double v3[3];
            for (int k = 0; k < 3; ++k) v3[k] = mu * d.dxi2[k] * fabs(ja[k][0] + ja[k][1] + ja[k][2]);
            visc = fmin(visc, d.dcfl * J / (v3[0] + v3[1] + v3[2]));
        }
    }
    __shared__ double sc[kThreads / 32], sv[kThreads / 32];
    for (int o = 16; o > 0; o >>= 1) {
        conv = fmin(conv, __shfl_down_sync(0xffffffffu, conv, o));
        visc = fmin(visc, __shfl_down_sync(0xffffffffu, visc, o));
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { sc[w] = conv; sv[w] = visc; }
    __syncthreads();
    if (w == 0) {
        conv = lane < kThreads / 32 ? sc[lane] : 1.0e300;
        visc = lane < kThreads / 32 ? sv[lane] : 1.0e300;
        for (int o = 16; o > 0; o >>= 1) {
            conv = fmin(conv, __shfl_down_sync(0xffffffffu, conv, o));
            visc = fmin(visc, __shfl_down_sync(0xffffffffu, visc, o));
        }
        if (lane == 0) {
            partials[2 * blockIdx.x] = conv;
            partials[2 * blockIdx.x + 1] = visc;
        }
    }
}

// Pass 2: one block folds the first nblocks partials of this call; the result goes to partials[0].
__global__ void k_dt_fold(double* partials, int nblocks) {
    double conv = 1.0e300, visc = 1.0e300;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
        conv = fmin(conv, partials[2 * b]);
        visc = fmin(visc, partials[2 * b + 1]);
    }
    __shared__ double sc[kThreads], sv[kThreads];
    sc[threadIdx.x] = conv;
    sv[threadIdx.x] = visc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sc[threadIdx.x] = fmin(sc[threadIdx.x], sc[threadIdx.x + s]);
            sv[threadIdx.x] = fmin(sv[threadIdx.x], sv[threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) partials[0] = sc[0] < sv[0] ? sc[0] : sv[0];
}

// Device address of g_partials, looked up once per device (cudaGetSymbolAddress with the device
// current); host code must never pass the symbol itself to a kernel. The cached address belongs to
// the device's context at the time of the lookup: after cudaDeviceReset it is stale, so a process
// that resets a device must not call dg_max_dt_noalloc on it again.
constexpr int kMaxDevices = 64;
std::mutex g_mutex;
double* g_partials_addr[kMaxDevices] = {};

int partials_address(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return h3d::fail(DG_ERR_NODEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return h3d::fail(DG_ERR_UNSUPPORTED, "device ordinal above 63");
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_partials_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_partials);
        if (e != cudaSuccess)
            return h3d::fail(DG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_partials_addr[dev] = static_cast<double*>(p);
    }
    *out = g_partials_addr[dev];
    return DG_OK;
}

}  // namespace

extern "C" {

int64_t dg_max_dt_noalloc_max_dof(void) { return static_cast<int64_t>(kMaxBlocks) * kNodesPerBlock; }

int dg_max_dt_noalloc(const double* q, const double* ja_xi, const double* ja_eta, const double* ja_zeta,
                      const double* jacobian, int64_t ndof, int order, int node_type, const dg_physics* phys,
                      double cfl, double dcfl, void* stream, double* dt) {
    if (!q || !ja_xi || !ja_eta || !ja_zeta || !jacobian || !phys || !dt)
        return h3d::fail(DG_ERR_INVALID, "null argument");
    if (ndof < 1) return h3d::fail(DG_ERR_INVALID, "ndof must be positive");
    if (ndof > dg_max_dt_noalloc_max_dof())
        return h3d::fail(DG_ERR_INVALID, "ndof exceeds the static scratch of dg_max_dt_noalloc (67,108,864 nodes)");
    if (order < 1 || order > 12) return h3d::fail(DG_ERR_INVALID, "polynomial order outside 1..12");
    if (node_type != DG_NODES_GAUSS && node_type != DG_NODES_GAUSS_LOBATTO)
        return h3d::fail(DG_ERR_INVALID, "unknown node type");
    if (!(phys->mach > 0.0)) return h3d::fail(DG_ERR_INVALID, "Mach number must be positive");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // An error left by the caller's own earlier work is reported as such, not as a failure here.
    cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess)
        return h3d::fail(DG_ERR_CUDA, std::string("dg_max_dt_noalloc: a CUDA error was pending before the call: ") +
                                          cudaGetErrorString(e));
    // The call synchronises the stream and copies dt to host memory, neither of which a stream
    // capture allows.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(s, &cap);
    if (e != cudaSuccess)
        return h3d::fail(DG_ERR_CUDA, std::string("dg_max_dt_noalloc: cudaStreamIsCapturing: ") + cudaGetErrorString(e));
    if (cap != cudaStreamCaptureStatusNone)
        return h3d::fail(DG_ERR_UNSUPPORTED, "dg_max_dt_noalloc cannot be called while its stream is being captured");
    double* partials = nullptr;
    int rc = partials_address(&partials);
    if (rc) return rc;
    DtConst d;
    d.ndof = ndof;
    d.cfl = cfl;
    d.dcfl = dcfl;
    const h3d::NodalStorage& ns = h3d::nodal_storage(node_type, order);
    for (int k = 0; k < 3; ++k) {
        d.dxi[k] = 1.0 / std::fabs(ns.x[1] - ns.x[0]);
        d.dxi2[k] = d.dxi[k] * d.dxi[k];
    }
    d.ns = phys->navier_stokes ? 1 : 0;
    d.gamma = 1.4;
    d.gm1 = 1.4 - 1.0;
    d.gammaM2 = d.gamma * (phys->mach * phys->mach);
    const double TRef = 520.0 * 5.0 / 9.0;
    d.S_div_TRef = (198.6 * 5.0 / 9.0) / TRef;
    d.TReNorm = TRef / TRef;
    const int nblocks = static_cast<int>((ndof + kNodesPerBlock - 1) / kNodesPerBlock);
    k_dt_partials<<<nblocks, kThreads, 0, s>>>(d, q, ja_xi, ja_eta, ja_zeta, jacobian, partials);
    e = cudaGetLastError();
    if (e == cudaSuccess) {
        k_dt_fold<<<1, kThreads, 0, s>>>(partials, nblocks);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(dt, partials, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return h3d::fail(DG_ERR_CUDA, std::string("dg_max_dt_noalloc: ") + cudaGetErrorString(e));
    return DG_OK;
}

}  // extern "C"
