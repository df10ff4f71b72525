// FP64 <-> FP32 conversions on the integer pipe.
//
// On GB300 the FP64 pipe runs at 1/64 of the FP32 rate and also executes the F2F conversion
// instructions. The mixed form converts every node value between the FP64 state and the FP32
// working precision several times per stage, so those conversions compete with the RK update's
// unavoidable FP64 multiply-adds. These functions build the IEEE-754 bit patterns with 32-bit integer
// operations instead, for the normal range of binary32; zeros keep their sign, and every other case
// (binary32 subnormals, overflow, infinities, NaN) goes to the hardware conversion, so the results
// equal __double2float_rn / the exact widening for every input.
//
// The cores work on raw bit patterns and compile for the host as well, so the rounding can be
// checked against the host's own conversion.
#pragma once
#include <cstdint>

#ifndef __CUDACC__
#define H3D_HD inline
#else
#define H3D_HD __host__ __device__ __forceinline__
#endif

namespace dg {

// binary64 (hi:lo words) -> binary32 bits, round to nearest even. Returns false when the input is
// outside the range handled here (|x| not in [2^-126, 2^128) and not a zero).
H3D_HD bool f32_bits_from_f64(uint32_t hi, uint32_t lo, uint32_t& out) {
    const uint32_t sgn = hi & 0x80000000u;
    const uint32_t e = (hi >> 20) & 0x7FFu;
    if (e == 0 && (hi & 0xFFFFFu) == 0 && lo == 0) {  // signed zero
        out = sgn;
        return true;
    }
    if (e < 1023u - 126u || e > 1023u + 127u) return false;
    const uint32_t m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);  // top 23 of the 52 mantissa bits
    const uint32_t rest = lo & 0x1FFFFFFFu;                  // the 29 bits rounded away
    uint32_t f = ((e - (1023u - 127u)) << 23) | m;
    const uint32_t half = 0x10000000u;
    f += (rest > half || (rest == half && (m & 1u))) ? 1u : 0u;  // a carry moves into the exponent (2^128 -> inf)
    out = sgn | f;
    return true;
}

// binary32 bits -> binary64 (hi:lo words), exact. Returns false for subnormals, infinities and NaN.
H3D_HD bool f64_bits_from_f32(uint32_t b, uint32_t& hi, uint32_t& lo) {
    const uint32_t e = (b >> 23) & 0xFFu;
    const uint32_t sgn = b & 0x80000000u;
    if (e == 0) {
        if ((b & 0x7FFFFFu) != 0) return false;
        hi = sgn;
        lo = 0;
        return true;
    }
    if (e == 0xFFu) return false;
    const uint32_t m = b & 0x7FFFFFu;
    hi = sgn | ((e + (1023u - 127u)) << 20) | (m >> 3);
    lo = m << 29;
    return true;
}

#ifdef __CUDACC__
__device__ __forceinline__ float to_f32(double x) {
    uint32_t f;
    if (f32_bits_from_f64(static_cast<uint32_t>(__double2hiint(x)), static_cast<uint32_t>(__double2loint(x)), f))
        return __uint_as_float(f);
    return __double2float_rn(x);
}

__device__ __forceinline__ double to_f64(float x) {
    uint32_t hi, lo;
    if (f64_bits_from_f32(__float_as_uint(x), hi, lo))
        return __hiloint2double(static_cast<int>(hi), static_cast<int>(lo));
    return static_cast<double>(x);
}

// Conversions into and out of the working precision R.
template <typename R>
__device__ __forceinline__ R from_f64(double x);
template <>
__device__ __forceinline__ float from_f64<float>(double x) { return to_f32(x); }
template <>
__device__ __forceinline__ double from_f64<double>(double x) { return x; }

__device__ __forceinline__ double widen(float x) { return to_f64(x); }
__device__ __forceinline__ double widen(double x) { return x; }
#endif

}  // namespace dg
