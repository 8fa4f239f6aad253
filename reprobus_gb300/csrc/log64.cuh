// log64.cuh — ln(x) to FP64 accuracy with 13 FP64-pipe instructions for
// positive normal x (the rate stage's logarithms of temperatures, pressures,
// water activity and weight fractions): on GB300 the library log costs about
// 30 FP64 operations, twice an exp.
//
// Method: P. T. P. Tang, "Table-driven implementation of the logarithm
// function in IEEE floating-point arithmetic", ACM TOMS 16(4), 1990, with
// N = 256 (log_table.h): x = 2^m y, y in [1, 2); F = 1 + j / 256 the nearest
// breakpoint (j = 0..256, from the first 9 mantissa bits); f = y - F exact;
// u = f / F as f * (1 / F) with |u| <= 2^-9;
//   ln x = (m LN2_HI + LOG64_HI[j]) + (m LN2_LO + LOG64_LO[j] + p(u)),
// the first sum exact (both terms multiples of 2^-42), p(u) = u + u^2 q(u)
// the degree-7 Taylor polynomial of ln(1 + u) (the next term below 2e-20 of
// u). y, F and m come from the bits; the FP64 instructions are the
// subtraction, the product by 1 / F, u^2, five FMAs of q, one of p, the two
// FMAs with m and the two final additions. Error: within 0.5 ulp but for x
// just below 1, where m ln 2 + ln F and ln(1 + u) partly cancel: 1.6 ulp
// there (tests/test_log64.py against long double, tests/test_gpu_log64.py
// against CUDA's log). Zero, negative, subnormal, inf and nan arguments
// return log(x).
#pragma once
#include "exp64.cuh"
#include "log_table.h"

namespace rpb {

__device__ __forceinline__ double log64(double x) {
    uint64_t b;
    memcpy(&b, &x, 8);
    const uint32_t hx = (uint32_t)(b >> 32);
    if (hx - 0x00100000u >= 0x7fe00000u) return log(x);  // not a positive normal
    const int m = (int)(hx >> 20) - 1023;
    const uint32_t mant_hi = hx & 0xfffffu;
    const int j = (int)((mant_hi + 0x800u) >> 12);  // 0..256: the nearest F
    const double y = e64_from(0x3ff00000u | mant_hi, (uint32_t)b);
    const double F = e64_from(0x3ff00000u + ((uint32_t)j << 12), 0u);
#ifdef __CUDA_ARCH__
    const double inv = __ldg(&LOG64_INV[j]), lhi = __ldg(&LOG64_HI[j]), llo = __ldg(&LOG64_LO[j]);
#else
    const double inv = LOG64_INV[j], lhi = LOG64_HI[j], llo = LOG64_LO[j];
#endif
    const double u = (y - F) * inv;
    const double u2 = u * u;
    double q = fma(u, 1. / 7., -1. / 6.);  // q(u) = -1/2 + u/3 - u^2/4 + u^3/5 - u^4/6 + u^5/7
    q = fma(u, q, 1. / 5.);
    q = fma(u, q, -1. / 4.);
    q = fma(u, q, 1. / 3.);
    q = fma(u, q, -1. / 2.);
    const double p = fma(u2, q, u);
    const double md = e64_int(m);
    const double hi = fma(md, LOG64_LN2_HI, lhi);
    const double lo = fma(md, LOG64_LN2_LO, llo);
    return hi + (lo + p);
}

}  // namespace rpb
