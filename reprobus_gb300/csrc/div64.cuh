// div64.cuh — a / b in FP64 with five FP64-pipe instructions after an
// approximate reciprocal: on GB300 the FP64 pipe issues 2 operations per
// clock per SM, and the IEEE division sequence takes about 9. For FP64-bound
// code (the rate stage); in the latency-bound solve kernels the extra range
// checks cost more than the FP64 instructions they save.
//
// Method: Newton-Raphson refinement of a reciprocal estimate r0 of b
// (r1 = r0 + r0 (1 - b r0): the relative error squares), the quotient
// q0 = a r1, and Markstein's correction q = q0 + r1 (a - b q0) (P. Markstein,
// "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Dev. 34(1), 1990), whose remainder a - b q0 one
// FMA gives exactly. With an estimate good to 2^-14 or better, q is within
// 2^-56 of a / b before its final rounding: the correctly rounded quotient
// but for a / b within 2^-56 of a rounding boundary, and at most one ulp
// away there (tests/test_div64.py, tests/test_gpu_div64.py).
//
// The estimate is the hardware's rcp.approx.ftz.f64 on the device; the host
// build (for the CPU checks) rounds 1 / b down to 20 bits instead. Operands
// outside the range where every intermediate stays normal (a or b zero,
// subnormal, beyond 2^+-1000, inf, nan, or a quotient beyond 2^+-1000) take
// the IEEE division.
#pragma once
#include "exp64.cuh"

namespace rpb {

// the IEEE division, out of line on the device: one call site per use of
// div64 instead of an inline copy of its sequence
#ifdef __CUDA_ARCH__
static __device__ __noinline__ double div64_ieee(double a, double b) { return a / b; }
#else
inline double div64_ieee(double a, double b) { return a / b; }
#endif

__device__ __forceinline__ double div64(double a, double b) {
    const int ea = (int)((e64_hi(a) >> 20) & 0x7ffu), eb = (int)((e64_hi(b) >> 20) & 0x7ffu);
    if (eb < 23 || eb > 2023 || ea < 23 || ea > 2023 || ea - eb > 1000 || eb - ea > 1000) return div64_ieee(a, b);
#ifdef __CUDA_ARCH__
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(b));
#else
    double r = 1.0 / b;
    uint64_t br;
    memcpy(&br, &r, 8);
    br &= ~((1ull << 32) - 1);
    memcpy(&r, &br, 8);
#endif
    r = fma(r, fma(-b, r, 1.0), r);
    const double q = a * r;
    return fma(r, fma(-b, q, a), q);
}

// sqrt(x) for positive normal x with six FP64-pipe instructions after the
// hardware's reciprocal square root estimate (rsqrt.approx.ftz.f64; the host
// build rounds 1 / sqrt(x) down to 20 bits): one Goldschmidt step refines
// s ~ sqrt(x) and h ~ 1 / (2 sqrt(x)) together, and the remainder x - s^2
// (exact in one FMA) corrects s (the same correction as div64's). Other
// arguments take the IEEE square root.
static __device__ __forceinline__ double sqrt64_ieee(double x) { return sqrt(x); }

__device__ __forceinline__ double sqrt64(double x) {
    if (e64_hi(x) - 0x00100000u >= 0x7fe00000u) return sqrt64_ieee(x);  // not a positive normal
#ifdef __CUDA_ARCH__
    double r;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
#else
    double r = 1.0 / sqrt(x);
    uint64_t br;
    memcpy(&br, &r, 8);
    br &= ~((1ull << 32) - 1);
    memcpy(&r, &br, 8);
#endif
    double s = x * r;
    double h = 0.5 * r;
    const double e = fma(-s, h, 0.5);
    s = fma(s, e, s);
    h = fma(h, e, h);
    return fma(fma(-s, s, x), h, s);
}

}  // namespace rpb
