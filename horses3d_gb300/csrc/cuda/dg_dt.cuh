// Device helpers of the CFL time step (MaxTimeStep) and the residual monitor (ComputeMaxResiduals,
// checkForNan), shared by the reduction kernels and by the update kernel that fuses them.
#pragma once
#include <cstdint>

#include "dg_convert.cuh"

namespace dg {

// ------------------------------------------------------------------------ reductions ----------
// Non-negative doubles order like their bit patterns, so atomicMin/atomicMax on the 64-bit image
// implement min/max reductions exactly (likewise non-negative floats and their 32-bit images).
__device__ __forceinline__ unsigned long long dbits(double x) { return static_cast<unsigned long long>(__double_as_longlong(x)); }
__device__ __forceinline__ unsigned int fbits(float x) { return __float_as_uint(x); }

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
__device__ __forceinline__ void dt_estimate_f(const DtConst32& d, float rho, float ru, float rv, float rw, float E,
                                              const R* jx, const R* je, const R* jz, R jac, float& conv, float& visc) {
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

// A working-precision value rounded to FP32 (the identity for FP32).
__device__ __forceinline__ float as_f32(float x) { return x; }
__device__ __forceinline__ float as_f32(double x) { return to_f32(x); }

// The estimate of the FP64 state Q (each value rounded to FP32 as the FP64 expressions' inputs).
template <typename R>
__device__ __forceinline__ void dt_estimate(const DtConst32& d, const double* Q, const R* jx, const R* je, const R* jz,
                                            R jac, float& conv, float& visc) {
    dt_estimate_f(d, to_f32(Q[0]), to_f32(Q[1]), to_f32(Q[2]), to_f32(Q[3]), to_f32(Q[4]), jx, je, jz, jac, conv, visc);
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

}  // namespace dg
