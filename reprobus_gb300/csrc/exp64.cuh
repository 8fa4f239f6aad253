// exp64.cuh — exp(y) to FP64 accuracy with four FP64-pipe instructions for
// |y| < 64 (the rate stage's Arrhenius, Troe and column-absorption
// exponentials): on GB300 the FP64 pipe issues 2 operations per clock per SM
// against 128 FP32 ones, and the library exp costs about 17 FP64 operations.
//
// Method: P. T. P. Tang, "Table-driven implementation of the exponential
// function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989, with a
// table of N = 512 entries (exp_table.h): y = k L + r, L = ln 2 / 512,
//   exp(y) = 2^(k >> 9) * T[k & 511] * exp(r),   |r| <= 0.51 L = 6.9e-4.
// Here
//   * k is picked in FP32 (y / L to within 0.01; no FP64 rounding step),
//     and k as a double is built from its bits;
//   * r1 = y - k L1 is exact (FMA; k L1 exact for |k| < 2^16); the rest of
//     the reduction, d = k (L - L1) <= 1.6e-10, enters in FP32;
//   * exp(r) - 1 = r1 + r1^2 / 2 (FP64, one FMA) + tail, with the FP32 tail
//     r1^3 (1/6 + r1 / 24) - d (1 + r1) (|tail| <= 5.3e-11, so its FP32
//     rounding is below 1e-17);
//   * the result T (1 + p) is one FMA, scaled by 2^(k >> 9) in its exponent
//     field.
// FP64 instructions: the two FMAs above, one add (p + tail) and the final
// FMA. The error is that of the final rounding, the table entry and the
// tail: at most about 1.5 ulp (tests/test_exp64.py checks the host build
// against long double, tests/test_gpu_exp64.py the device code against
// CUDA's exp). Below -745.2 it returns 0 (as exp does); elsewhere outside
// |y| < 64 (and for NaN, inf) it returns exp(y).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#ifndef __CUDACC__
#ifndef __device__
#define __device__
#endif
#ifndef __forceinline__
#define __forceinline__ inline
#endif
#endif

#include "exp_table.h"

namespace rpb {

__device__ __forceinline__ uint32_t e64_hi(double v) {
    uint64_t b;
    memcpy(&b, &v, 8);
    return (uint32_t)(b >> 32);
}
__device__ __forceinline__ double e64_from(uint32_t hi, uint32_t lo) {
    const uint64_t b = ((uint64_t)hi << 32) | lo;
    double d;
    memcpy(&d, &b, 8);
    return d;
}
__device__ __forceinline__ float e64_f32(uint32_t f) {
    float r;
    memcpy(&r, &f, 4);
    return r;
}
__device__ __forceinline__ uint32_t e64_bits(float v) {
    uint32_t f;
    memcpy(&f, &v, 4);
    return f;
}
__device__ __forceinline__ int e64_clz(uint32_t a) {
#ifdef __CUDA_ARCH__
    return __clz((int)a);
#else
    return __builtin_clz(a);
#endif
}

// double -> float by truncation for |v| in [2^-126, 2^128) (else 0; the
// callers pass |v| < 64 or the small reduced argument)
__device__ __forceinline__ float e64_to_f32(double v) {
    uint64_t b;
    memcpy(&b, &v, 8);
    const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    const int E = (int)((hi >> 20) & 0x7ffu);
    if (E <= 896) return 0.f;
    return e64_f32((hi & 0x80000000u) | ((uint32_t)(E - 896) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
}

// float -> double, exact for normal floats and zero (subnormals flush to zero)
__device__ __forceinline__ double e64_to_f64(float z) {
    const uint32_t f = e64_bits(z);
    const uint32_t E = (f >> 23) & 0xffu, m = f & 0x7fffffu;
    if (E == 0) return e64_from(f & 0x80000000u, 0u);
    return e64_from((f & 0x80000000u) | ((E + 896u) << 20) | (m >> 3), m << 29);
}

// a small integer (|k| < 2^20) as a double, from its bits
__device__ __forceinline__ double e64_int(int k) {
    if (k == 0) return 0.;
    const uint32_t s = k < 0 ? 0x80000000u : 0u;
    const uint32_t a = (uint32_t)(k < 0 ? -k : k);
    const int e = 31 - e64_clz(a);  // leading bit
    return e64_from(s | ((uint32_t)(1023 + e) << 20) | ((a << (20 - e)) & 0xfffffu), 0u);
}

__device__ __forceinline__ double exp64(double y) {
    const uint32_t hy = e64_hi(y);
    if ((hy & 0x7ff00000u) >= 0x40500000u) {  // |y| >= 64, inf, nan
        // exp(y) rounds to 0 below -745.2 (the column absorption terms of
        // J(NO) deep in the atmosphere): no library call for those
        if (y < -745.2) return 0.;
        return exp(y);
    }
    // k = rint(y / L) in FP32 (|y / L| < 2^22: the 1.5 2^23 shift rounds it)
    const float kf = fmaf(e64_to_f32(y), EXP64_INVF, 12582912.f);
    const int k = (int)e64_bits(kf) - (int)e64_bits(12582912.f);
    const double r1 = fma(e64_int(k), -EXP64_L1, y);
    // r1 / 2 by the exponent field (|r1| below 2^-1021: its square is nothing)
    const uint32_t hr = e64_hi(r1);
    uint64_t br;
    memcpy(&br, &r1, 8);
    const double r1h = (hr & 0x7ff00000u) > 0x00100000u ? e64_from(hr - 0x00100000u, (uint32_t)br) : 0.;
    const double p = fma(r1, r1h, r1);  // r1 + r1^2 / 2
    const float rf = e64_to_f32(r1);
    const float d = (float)k * EXP64_L2F;
    const float tail = fmaf(rf * rf * rf, fmaf(rf, 1.f / 24.f, 1.f / 6.f), -fmaf(d, rf, d));
#ifdef __CUDA_ARCH__
    const double t = __ldg(&EXP64_TAB[k & (EXP64_N - 1)]);
#else
    const double t = EXP64_TAB[k & (EXP64_N - 1)];
#endif
    const double res = fma(t, p + e64_to_f64(tail), t);
    // times 2^(k >> 9): res is in [0.99, 2.01), the result normal for |y| < 64
    uint64_t bres;
    memcpy(&bres, &res, 8);
    bres += (uint64_t)(int64_t)(k >> 9) << 52;
    double out;
    memcpy(&out, &bres, 8);
    return out;
}

}  // namespace rpb
