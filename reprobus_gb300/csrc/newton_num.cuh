// newton_num.cuh — number-format helpers of the Newton solver, written with
// integer operations on the IEEE-754 fields so that no FP64-pipe conversion
// instruction is spent on them (FP64 throughput on GB300 is 1/64 of FP32).
//
//   nt_exp_hi(v)         biased exponent field of |v| in place (high word of v
//                        & 0x7ff00000)
//   nt_scale<T>(e, fh)   2^(E-1023), E = max(e, fh) >> 20: the power of two
//                        s <= max(|x|, floor) < 2 s, as T (exact)
//   nt_rscale<T>(e, fh)  1/s (exact)
//   nt_cvt<T>(v)         double -> T; for float the mantissa is truncated and
//                        magnitudes below 2^-126 flush to zero (the Jacobian
//                        and the right-hand side only need FP32 accuracy)
//   nt_widen(z)          T -> double, exact for normal floats
#pragma once
#include <cstdint>
#include <cstring>

// compiler-level memory fence: no load or store is moved across it, so the
// generated factorisation keeps each row's loads in that row
#ifdef __CUDA_ARCH__
#define NT_FENCE() asm volatile("" ::: "memory")
#else
#define NT_FENCE() ((void)0)
#endif

namespace rpb {

__device__ __forceinline__ int nt_exp_hi(double v) {
    uint64_t b;
    memcpy(&b, &v, 8);
    return (int)(b >> 32) & 0x7ff00000;
}

__device__ __forceinline__ double nt_f64_from_hi(uint32_t hi) {
    const uint64_t b = (uint64_t)hi << 32;
    double d;
    memcpy(&d, &b, 8);
    return d;
}

__device__ __forceinline__ float nt_f32_from_bits(uint32_t f) {
    float r;
    memcpy(&r, &f, 4);
    return r;
}

// float exponent field of the power of two with double exponent field E,
// clamped to the normal float range
__device__ __forceinline__ uint32_t nt_f32_exp(int E) {
    int f = E - 896;
    f = f < 1 ? 1 : (f > 254 ? 254 : f);
    return (uint32_t)f << 23;
}

template <typename T>
__device__ __forceinline__ T nt_scale(int e, int fh);
template <>
__device__ __forceinline__ double nt_scale<double>(int e, int fh) {
    return nt_f64_from_hi((uint32_t)(e > fh ? e : fh));
}
template <>
__device__ __forceinline__ float nt_scale<float>(int e, int fh) {
    return nt_f32_from_bits(nt_f32_exp((e > fh ? e : fh) >> 20));
}

template <typename T>
__device__ __forceinline__ T nt_rscale(int e, int fh);
template <>
__device__ __forceinline__ double nt_rscale<double>(int e, int fh) {
    return nt_f64_from_hi((uint32_t)(0x7fe00000 - (e > fh ? e : fh)));
}
template <>
__device__ __forceinline__ float nt_rscale<float>(int e, int fh) {
    return nt_f32_from_bits(nt_f32_exp(2046 - ((e > fh ? e : fh) >> 20)));
}

template <typename T>
__device__ __forceinline__ T nt_cvt(double v);
template <>
__device__ __forceinline__ double nt_cvt<double>(double v) {
    return v;
}
template <>
__device__ __forceinline__ float nt_cvt<float>(double v) {
    uint64_t b;
    memcpy(&b, &v, 8);
    const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    const uint32_t sign = hi & 0x80000000u;
    const int E = (int)((hi >> 20) & 0x7ffu);
    uint32_t f;
    if (E <= 896)
        f = sign;  // below the float normal range: +-0
    else if (E >= 1151)
        f = sign | 0x7f800000u | ((E == 2047 && ((hi & 0xfffffu) | lo)) ? 0x400000u : 0u);  // inf / nan
    else
        f = sign | ((uint32_t)(E - 896) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    return nt_f32_from_bits(f);
}

// Quotients of the generated equations. FP64 (the residual; the FP64
// solver's Jacobian): the hardware's reciprocal estimate, one Newton-Raphson
// step and Markstein's correction (P. Markstein, IBM J. Res. Dev. 34(1),
// 1990) with no range test: five FP64 instructions against the IEEE
// sequence's nine and its slow-path branch. For operands whose magnitudes
// lie in 2^+-1000, as the chemistry's do, the quotient is the IEEE one but
// for a / b within 2^-56 of a rounding boundary (one ulp there); a zero
// divisor or an infinite dividend gives NaN where IEEE gives an infinity,
// which fails the cell all the same. FP32 (the mixed solver's Jacobian, which
// only steers the iteration): the fast division, within 2 ulp for divisors
// below 2^126. The host build (CPU checks of the generated code) divides.
template <typename T>
__device__ __forceinline__ T nt_div(T a, T b);
template <>
__device__ __forceinline__ double nt_div<double>(double a, double b) {
#ifdef __CUDA_ARCH__
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(b));
    r = fma(r, fma(-b, r, 1.0), r);
    const double q = a * r;
    return fma(r, fma(-b, q, a), q);
#else
    return a / b;
#endif
}
template <>
__device__ __forceinline__ float nt_div<float>(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fdividef(a, b);
#else
    return a / b;
#endif
}

// Pivot reciprocals of the factorisation (|p| >= the pivot guard): FP64 as
// nt_div(1, p); FP32 the hardware's approximate reciprocal, within 1 ulp
// (a pivot beyond 2^126 would give 0 and fail its cell; the scaled pivots
// are far below that).
template <typename T>
__device__ __forceinline__ T nt_rcp(T p);
template <>
__device__ __forceinline__ double nt_rcp<double>(double p) {
    return nt_div<double>(1.0, p);
}
template <>
__device__ __forceinline__ float nt_rcp<float>(float p) {
#ifdef __CUDA_ARCH__
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(p));
    return r;
#else
    return 1.0f / p;
#endif
}

__device__ __forceinline__ double nt_widen(double z) { return z; }
__device__ __forceinline__ double nt_widen(float z) {
    uint32_t f;
    memcpy(&f, &z, 4);
    const uint32_t sign = f & 0x80000000u, E = (f >> 23) & 0xffu, m = f & 0x7fffffu;
    uint64_t b;
    if (E == 0)
        b = (uint64_t)sign << 32;  // zero (subnormals flush to zero)
    else if (E == 255)
        b = ((uint64_t)(sign | 0x7ff00000u | (m >> 3)) << 32) | ((uint64_t)m << 29);
    else
        b = ((uint64_t)(sign | ((E + 896u) << 20) | (m >> 3)) << 32) | (uint64_t)(m << 29);
    double d;
    memcpy(&d, &b, 8);
    return d;
}

}  // namespace rpb
