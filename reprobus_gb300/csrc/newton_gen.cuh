// newton_gen.cuh — GENERATED by reprobus_gb300/codegen/gen_newton.py; do not edit.
//
// Residual, scaled analytic Jacobian and sparse Crout LU of the chemistry step
// equations (fixed point of one pass of src/reprobus_l137_20230723.f:1350-2372,
// in the Jacobi form described in the generator). Unknowns x[0..41] = ck(1..42),
// x[42..56] = cc(1..15).
// Jacobian: 401 structural non-zeros (day|night|diagonal), 19 of them constant
// diagonal entries; stored A entries 382; off-diagonal U~ entries 270; LU updates 1064;
// shared-memory slots per cell 382.
// elimination order (Markowitz, refined): [6, 40, 32, 3, 17, 38, 33, 11, 29, 36, 31, 26, 39, 37, 19, 15, 35, 54, 5, 0, 51, 25, 13, 34, 30, 24, 42, 9, 7, 4, 41, 22, 21, 1, 8, 14, 56, 18, 16, 23, 55, 28, 27, 20, 12, 2, 48, 45, 10, 44, 53, 50, 43, 47, 46, 49, 52]
#pragma once
#ifndef __CUDACC__
#define __device__
#define __forceinline__ inline
#endif
#include "newton_num.cuh"

namespace rpb {
constexpr int NT_NX = 57;
constexpr int NT_NNZ = 401;
constexpr int NT_NA = 382;        // stored entries of A (the Jacobian)
constexpr int NT_NSLOT = 382;     // shared-memory matrix slots per cell
constexpr int NT_NUPD = 1064;     // multiply-adds of the factorisation
constexpr int NT_PERM[57] = {6, 40, 32, 3, 17, 38, 33, 11, 29, 36, 31, 26, 39, 37, 19, 15, 35, 54, 5, 0, 51, 25, 13, 34, 30, 24, 42, 9, 7, 4, 41, 22, 21, 1, 8, 14, 56, 18, 16, 23, 55, 28, 27, 20, 12, 2, 48, 45, 10, 44, 53, 50, 43, 47, 46, 49, 52};  // elimination position k holds unknown NT_PERM[k]
constexpr int NT_A_I[382] = {6, 6, 6, 6, 6, 6, 6, 6, 6, 6, 6, 40, 40, 40, 40, 40, 40, 40, 32, 32, 3, 3, 3, 3, 3, 17, 17, 17, 17, 17, 38, 38, 33, 33, 29, 29, 29, 29, 36, 36, 36, 31, 31, 26, 26, 26, 26, 26, 26, 26, 39, 39, 37, 37, 37, 19, 19, 19, 19, 19, 15, 15, 15, 15, 15, 15, 35, 35, 54, 54, 54, 5, 5, 5, 5, 5, 0, 0, 51, 25, 25, 25, 25, 25, 25, 25, 25, 13, 13, 13, 13, 13, 13, 34, 34, 30, 30, 24, 24, 42, 9, 9, 9, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 7, 4, 4, 4, 4, 4, 4, 4, 4, 41, 41, 22, 22, 22, 22, 22, 22, 22, 22, 22, 22, 22, 22, 22, 22, 22, 22, 22, 22, 22, 22, 22, 22, 22, 22, 22, 21, 21, 21, 21, 1, 1, 1, 1, 8, 8, 8, 8, 8, 8, 14, 14, 14, 14, 14, 14, 14, 14, 14, 14, 56, 56, 56, 56, 56, 18, 18, 18, 18, 18, 18, 18, 18, 16, 16, 16, 23, 23, 23, 23, 23, 23, 23, 23, 23, 23, 23, 23, 23, 55, 55, 55, 55, 55, 28, 28, 28, 28, 28, 28, 28, 27, 27, 27, 27, 27, 27, 27, 27, 27, 27, 27, 27, 20, 20, 20, 20, 20, 20, 20, 20, 20, 20, 20, 20, 20, 20, 20, 20, 20, 20, 12, 12, 12, 12, 12, 12, 12, 12, 12, 12, 12, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 48, 48, 48, 48, 48, 48, 48, 48, 48, 45, 45, 45, 45, 45, 45, 44, 44, 44, 44, 44, 44, 44, 44, 44, 44, 44, 44, 44, 53, 53, 53, 53, 53, 53, 53, 53, 53, 53, 50, 50, 50, 50, 50, 50, 50, 50, 50, 43, 43, 43, 43, 43, 43, 43, 43, 43, 43, 43, 43, 43, 43, 43, 43, 43, 43, 43, 43, 43, 43, 43, 43, 43, 43, 47, 47, 47, 47, 47, 47, 47, 47, 47, 47, 47, 47, 47, 46, 46, 46, 46, 46, 46, 49, 49, 49, 49, 49, 49, 49, 52, 52, 52, 52, 52, 52, 52, 52, 52, 52, 52, 52, 52, 52};
constexpr int NT_A_J[382] = {32, 38, 33, 36, 31, 35, 34, 30, 42, 12, 43, 38, 39, 37, 42, 41, 18, 43, 32, 42, 0, 51, 42, 4, 49, 17, 5, 12, 48, 44, 38, 42, 33, 42, 29, 28, 43, 47, 36, 42, 43, 31, 42, 26, 25, 14, 18, 12, 53, 52, 39, 42, 37, 42, 43, 19, 2, 48, 45, 53, 15, 13, 14, 12, 44, 52, 35, 43, 20, 48, 46, 54, 5, 12, 2, 48, 0, 42, 49, 19, 25, 18, 12, 2, 45, 53, 47, 13, 12, 2, 48, 45, 52, 34, 43, 30, 42, 24, 52, 46, 9, 53, 52, 26, 25, 13, 14, 55, 28, 48, 45, 53, 43, 47, 46, 49, 52, 19, 5, 13, 4, 12, 2, 48, 43, 41, 43, 32, 17, 33, 36, 31, 26, 15, 35, 13, 34, 30, 24, 42, 9, 1, 14, 27, 12, 48, 45, 44, 53, 43, 47, 52, 21, 48, 43, 47, 42, 1, 44, 43, 8, 27, 45, 44, 50, 43, 13, 14, 18, 12, 2, 45, 44, 43, 47, 52, 42, 1, 45, 44, 43, 25, 42, 14, 18, 27, 50, 43, 47, 16, 43, 47, 26, 19, 25, 42, 18, 27, 48, 45, 53, 50, 43, 47, 52, 8, 45, 43, 47, 46, 29, 56, 28, 43, 47, 49, 52, 29, 42, 1, 56, 28, 27, 45, 44, 50, 43, 49, 52, 17, 19, 54, 5, 0, 51, 13, 42, 4, 21, 48, 45, 44, 53, 43, 47, 49, 52, 5, 25, 13, 1, 14, 27, 12, 44, 43, 47, 52, 29, 42, 4, 1, 16, 55, 27, 12, 2, 43, 47, 28, 20, 48, 45, 53, 47, 46, 49, 52, 55, 44, 43, 47, 46, 49, 1, 14, 28, 12, 2, 48, 45, 53, 43, 47, 46, 49, 52, 23, 27, 48, 45, 53, 43, 47, 46, 49, 52, 27, 48, 45, 53, 43, 47, 46, 49, 52, 29, 25, 42, 4, 21, 1, 8, 14, 56, 18, 16, 55, 28, 27, 12, 2, 48, 45, 44, 53, 50, 43, 47, 46, 49, 52, 8, 16, 55, 27, 45, 44, 53, 50, 43, 47, 46, 49, 52, 7, 55, 44, 43, 47, 49, 28, 48, 45, 53, 47, 46, 52, 22, 1, 14, 28, 12, 2, 48, 45, 53, 43, 47, 46, 49, 52};
constexpr int NT_NCONST = 19;
constexpr int NT_CONST_I[19] = {3, 6, 7, 10, 11, 20, 22, 23, 40, 42, 44, 45, 46, 49, 50, 51, 54, 55, 56};  // constant diagonal entries
constexpr double NT_CONST_V[19] = {1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0};

// per-cell constants of the equations
struct NtFix {
    double o2, n2, h2, co2, hnm, parthno3, parth2o, parthcl, parthbr;
    double rain_hno3, rain_hcl, rain_hbr, rain_h2o2, dt;
};
template <typename T> struct NtFixT {
    T o2, n2, h2, co2, hnm, parthno3, parth2o, parthcl, parthbr;
    T rain_hno3, rain_hcl, rain_hbr, rain_h2o2, dt;
};


// residual R(x), day equations (FP64; K/tj/het/ck0/x: pointers or views)
template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>
__device__ __forceinline__ void nt_residual_day(const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {
    R[0] = -ck0[0] + x[0]*(F.dt*(tj[J_n2o] + x[42]*(K[K_b38] + K[K_b39])) + T(1));
    R[1] = -ck0[1] + x[1]*(F.dt*(K[K_c1a]*x[42] + K[K_c1b]*x[42] + K[K_c1c]*x[42] + K[K_c2]*x[43] + K[K_d5]*x[44]) + T(1));
    const T dr2_c0 = x[29]*x[43];
    R[2] = -F.dt*(F.h2*K[K_a19]*x[43] + F.parthcl*K[K_d11]*x[12]*x[43] + F.parthno3*K[K_b27]*x[43]*x[4] + K[K_a30]*x[16]*x[43] + K[K_a31]*(x[43]*x[43]) + K[K_c17a]*dr2_c0 + K[K_c17b]*dr2_c0 + K[K_c2]*x[1]*x[43] + K[K_c8]*x[27]*x[43] + x[47]*(K[K_a17]*x[43] + T(1.6e-12)*x[55])) - ck0[2] + x[2]*(F.dt*F.parth2o*(K[K_a1et]*x[42] + tj[J_h2o]) + T(1));
    R[3] = -T(2)*F.dt*K[K_b39]*x[0]*x[42] + F.dt*(F.rain_hno3*x[4] + T(2)*K[K_b6]*x[49]*x[51]) - ck0[3] + x[3];
    R[4] = -F.dt*(K[K_b22]*x[43]*x[48] + het[0]*x[13]*x[2] + het[1]*x[12]*x[13] + T(2)*het[2]*x[2]*x[5] + het[3]*x[12]*x[5] + het[5]*x[19]*x[2]) - ck0[4] + x[4]*(F.dt*(F.parthno3*(K[K_b27]*x[43] + tj[J_hno3]) + F.rain_hno3) + T(1));
    R[5] = -F.dt*K[K_b12]*x[48]*x[54] - ck0[5] + x[5]*(F.dt*(F.hnm*K[K_b32] + het[2]*x[2] + het[3]*x[12] + tj[J_n2o5]) + T(1));
    const T dr6_c0 = T(3)*x[42];
    R[6] = F.dt*F.rain_hcl*x[12] - F.dt*(x[30]*(K[K_d90]*dr6_c0 + T(3)*tj[J_cfc11]) + x[31]*(T(2)*K[K_d91]*x[42] + T(2)*tj[J_cfc12]) + x[32]*(K[K_d92]*dr6_c0 + T(3)*tj[J_cfc113]) + x[33]*(T(4)*K[K_d93]*x[42] + T(4)*tj[J_ccl4]) + x[34]*(T(3)*K[K_d94]*x[43] + T(3)*tj[J_ch3ccl3]) + x[35]*(K[K_d95]*x[43] + tj[J_ch3cl]) + x[36]*(K[K_d96]*x[42] + K[K_d97]*x[43] + tj[J_hcfc22]) + x[38]*(K[K_e52]*x[42] + tj[J_h1211])) - ck0[6] + x[6];
    R[9] = -F.dt*K[K_e5a]*x[52]*x[53] - ck0[9] + x[9]*(F.dt*tj[J_oclo] + T(1));
    R[10] = -ck0[10] + x[10];
    R[11] = -ck0[11] + x[11];
    R[12] = -F.dt*(K[K_d9]*x[43]*x[52] + x[44]*(F.h2*K[K_d6] + K[K_c10]*x[27] + K[K_d5]*x[1] + K[K_d7]*x[47])) - ck0[12] + x[12]*(F.dt*(F.parthcl*(K[K_d11]*x[43] + tj[J_hcl]) + F.rain_hcl + het[1]*x[13] + het[3]*x[5] + het[4]*x[14] + het[6]*x[25]) + T(1));
    R[13] = -F.dt*K[K_d31]*x[48]*x[52] - ck0[13] + x[13]*(F.dt*(K[K_d32]*x[45] + het[0]*x[2] + het[1]*x[12] + tj[J_clono2_cl] + tj[J_clono2_clo]) + T(1));
    R[14] = -F.dt*(K[K_d33]*x[47]*x[52] + het[0]*x[13]*x[2]) - ck0[14] + x[14]*(F.dt*(K[K_d34]*x[43] + K[K_d35]*x[45] + K[K_d37]*x[44] + het[4]*x[12] + het[8]*x[18] + tj[J_hocl]) + T(1));
    R[15] = -F.dt*(K[K_d37]*x[14]*x[44] + K[K_d62]*(x[52]*x[52]) + het[1]*x[12]*x[13] + het[4]*x[12]*x[14]) - ck0[15] + x[15]*(F.dt*tj[J_cl2] + T(1));
    R[16] = -F.dt*K[K_a27]*(x[47]*x[47]) - ck0[16] + x[16]*(F.dt*(F.rain_h2o2 + K[K_a30]*x[43] + tj[J_h2o2]) + T(1));
    R[17] = -F.dt*(K[K_d36]*x[44]*x[48] + het[3]*x[12]*x[5]) - ck0[17] + x[17]*(F.dt*tj[J_clno2] + T(1));
    R[18] = -F.dt*(K[K_c19]*x[27]*x[50] + K[K_e7]*x[47]*x[50]) - ck0[18] + x[18]*(F.dt*(F.parthbr*(K[K_e11]*x[43] + K[K_e9]*x[42] + tj[J_hbr]) + F.rain_hbr + het[7]*x[25] + het[8]*x[14]) + T(1));
    R[19] = -F.dt*K[K_e13]*x[48]*x[53] - ck0[19] + x[19]*(F.dt*(K[K_e8]*x[45] + het[5]*x[2] + tj[J_brono2]) + T(1));
    const T dr20_c0 = F.parthno3*x[4];
    R[20] = F.dt*(T(2)*K[K_b6]*x[49]*x[51] + x[48]*(T(2)*K[K_b12]*x[54] + K[K_b22]*x[43] + K[K_b23]*x[47] + K[K_d31]*x[52] + K[K_d36]*x[44] + K[K_e13]*x[53])) - F.dt*(K[K_b27]*dr20_c0*x[43] + T(2)*K[K_b39]*x[0]*x[42] + K[K_d32]*x[13]*x[45] + K[K_e8]*x[19]*x[45] + dr20_c0*tj[J_hno3] + tj[J_brono2]*x[19] + tj[J_clno2]*x[17] + x[13]*(tj[J_clono2_cl] + tj[J_clono2_clo]) + x[21]*(F.hnm*K[K_b24] + K[K_b28]*x[43] + tj[J_hno4]) + x[5]*(T(2)*F.hnm*K[K_b32] + T(2)*tj[J_n2o5])) - ck0[20] + x[20];
    R[21] = -F.dt*K[K_b23]*x[47]*x[48] - ck0[21] + x[21]*(F.dt*(F.hnm*K[K_b24] + K[K_b28]*x[43] + tj[J_hno4]) + T(1));
    const T dr22_c0 = T(2)*x[52];
    const T dr22_c1 = T(3)*x[42];
    R[22] = F.dt*(x[44]*(F.h2*K[K_d6] + K[K_c10]*x[27] + K[K_d36]*x[48] + K[K_d37]*x[14] + K[K_d5]*x[1] + K[K_d7]*x[47]) + x[52]*(K[K_d31]*x[48] + K[K_d33]*x[47] + K[K_d60]*dr22_c0 + K[K_d62]*dr22_c0 + K[K_d9]*x[43] + K[K_e5a]*x[53] + K[K_e5c]*x[53])) - F.dt*(F.parthcl*x[12]*(K[K_d11]*x[43] + tj[J_hcl]) + tj[J_brcl]*x[26] + T(2)*tj[J_cl2]*x[15] + tj[J_clno2]*x[17] + tj[J_oclo]*x[9] + x[13]*(K[K_d32]*x[45] + tj[J_clono2_cl] + tj[J_clono2_clo]) + x[14]*(K[K_d34]*x[43] + K[K_d35]*x[45] + tj[J_hocl]) + x[24]*(T(2)*F.hnm*K[K_d61] + T(2)*tj[J_cl2o2]) + x[30]*(K[K_d90]*dr22_c1 + T(3)*tj[J_cfc11]) + x[31]*(T(2)*K[K_d91]*x[42] + T(2)*tj[J_cfc12]) + x[32]*(K[K_d92]*dr22_c1 + T(3)*tj[J_cfc113]) + x[33]*(T(4)*K[K_d93]*x[42] + T(4)*tj[J_ccl4]) + x[34]*(T(3)*K[K_d94]*x[43] + T(3)*tj[J_ch3ccl3]) + x[35]*(K[K_d95]*x[43] + tj[J_ch3cl]) + x[36]*(K[K_d96]*x[42] + K[K_d97]*x[43] + tj[J_hcfc22])) - ck0[22] + x[22];
    R[23] = F.dt*(K[K_c19]*x[27]*x[50] + K[K_e7]*x[47]*x[50] + x[53]*(K[K_e13]*x[48] + K[K_e15]*x[47] + K[K_e5c]*x[52])) - F.dt*(F.parthbr*x[18]*(K[K_e11]*x[43] + K[K_e9]*x[42] + tj[J_hbr]) + K[K_e16]*x[25]*x[45] + K[K_e8]*x[19]*x[45] + T(2)*het[7]*x[18]*x[25] + tj[J_brcl]*x[26] + tj[J_brono2]*x[19] + tj[J_hobr]*x[25]) - ck0[23] + x[23];
    R[24] = -F.dt*K[K_d60]*(x[52]*x[52]) - ck0[24] + x[24]*(F.dt*(F.hnm*K[K_d61] + tj[J_cl2o2]) + T(1));
    R[25] = -F.dt*(K[K_e15]*x[47]*x[53] + het[5]*x[19]*x[2]) - ck0[25] + x[25]*(F.dt*(K[K_e16]*x[45] + het[6]*x[12] + het[7]*x[18] + tj[J_hobr]) + T(1));
    R[26] = -F.dt*(K[K_e5c]*x[52]*x[53] + het[6]*x[12]*x[25] + het[8]*x[14]*x[18]) - ck0[26] + x[26]*(F.dt*tj[J_brcl] + T(1));
    R[28] = -F.dt*(F.o2*K[K_c4]*x[56] + K[K_c17a]*x[29]*x[43]) - ck0[28] + x[28]*(F.dt*(T(2)*K[K_c14]*x[28] + K[K_c18]*x[52] + K[K_c5]*x[49] + K[K_c7]*x[47]) + T(1));
    R[29] = -F.dt*K[K_c7]*x[28]*x[47] - ck0[29] + x[29]*(F.dt*(K[K_c17a]*x[43] + K[K_c17b]*x[43] + tj[J_ch3o2h]) + T(1));
    R[30] = -ck0[30] + x[30]*(F.dt*(K[K_d90]*x[42] + tj[J_cfc11]) + T(1));
    R[31] = -ck0[31] + x[31]*(F.dt*(K[K_d91]*x[42] + tj[J_cfc12]) + T(1));
    R[32] = -ck0[32] + x[32]*(F.dt*(K[K_d92]*x[42] + tj[J_cfc113]) + T(1));
    R[33] = -ck0[33] + x[33]*(F.dt*(K[K_d93]*x[42] + tj[J_ccl4]) + T(1));
    R[34] = -ck0[34] + x[34]*(F.dt*(K[K_d94]*x[43] + tj[J_ch3ccl3]) + T(1));
    R[35] = -ck0[35] + x[35]*(F.dt*(K[K_d95]*x[43] + tj[J_ch3cl]) + T(1));
    R[36] = -ck0[36] + x[36]*(F.dt*(K[K_d96]*x[42] + K[K_d97]*x[43] + tj[J_hcfc22]) + T(1));
    R[37] = -ck0[37] + x[37]*(F.dt*(K[K_e50]*x[42] + K[K_e51]*x[43] + tj[J_ch3br]) + T(1));
    R[38] = -ck0[38] + x[38]*(F.dt*(K[K_e52]*x[42] + tj[J_h1211]) + T(1));
    R[39] = -ck0[39] + x[39]*(F.dt*(K[K_e53]*x[42] + tj[J_h1301]) + T(1));
    R[40] = F.dt*F.rain_hbr*x[18] - F.dt*(x[37]*(K[K_e50]*x[42] + K[K_e51]*x[43] + tj[J_ch3br]) + x[38]*(K[K_e52]*x[42] + tj[J_h1211]) + x[39]*(K[K_e53]*x[42] + tj[J_h1301]) + x[41]*(T(2)*K[K_e54]*x[43] + T(2)*tj[J_ch2br2])) - ck0[40] + x[40];
    R[41] = -ck0[41] + x[41]*(F.dt*(K[K_e54]*x[43] + tj[J_ch2br2]) + T(1));
    R[42] = nt_div<T>(-tj[J_o3_o1d]*x[46], F.n2*K[K_hk4] + F.o2*K[K_hk5]) + x[42];
    R[56] = nt_div<T>(-x[1]*(K[K_c1a]*x[42] + K[K_c2]*x[43] + K[K_d5]*x[44]), F.o2*K[K_c4] + K[K_c3]*x[45]) + x[56];
    const T D_ch3o = nt_div<T>(K[K_c1b]*x[1]*x[42] + tj[J_ch3o2h]*x[29] + x[28]*(T(2)*K[K_c14]*x[28] + K[K_c18]*x[52] + K[K_c5]*x[49]), F.o2*K[K_c15]);
    R[27] = -F.dt*(D_ch3o*F.o2*K[K_c15] + K[K_c17b]*x[29]*x[43] + K[K_c1c]*x[1]*x[42] + K[K_c3]*x[45]*x[56]) - ck0[27] + x[27]*(F.dt*(K[K_c10]*x[44] + K[K_c19]*x[50] + K[K_c8]*x[43] + K[K_c9]*x[45] + tj[J_ch2o_co] + tj[J_ch2o_hco]) + T(1));
    const T D_hco = nt_div<T>(x[27]*(K[K_c10]*x[44] + K[K_c19]*x[50] + K[K_c8]*x[43] + K[K_c9]*x[45] + tj[J_ch2o_hco]), F.o2*K[K_c12]);
    R[8] = -F.dt*(D_hco*F.o2*K[K_c12] + F.co2*tj[J_co2] + tj[J_ch2o_co]*x[27]) - ck0[8] + x[8]*(F.dt*K[K_a36]*x[43] + T(1));
    const T D_r1 = nt_div<T>(K[K_a2]*x[55] + K[K_a6]*x[43] + K[K_a6b]*x[47] + K[K_b4]*x[49] + K[K_d2]*x[44] + tj[J_o3_o1d] + tj[J_o3_o3p], F.o2*K[K_hk2]);
    R[45] = -D_r1*x[46] + x[45];
    R[46] = x[46] + nt_div<T>(-x[7], D_r1 + T(1));
    const T D_r4 = nt_div<T>(F.h2*K[K_a19] + K[K_a36]*x[8] + K[K_a5]*x[45], F.o2*K[K_a1] + K[K_a2]*x[46] + T(8.049999999999999e-11)*x[47]);
    R[55] = -D_r4*x[43] + x[55];
    const T D_r7 = nt_div<T>(tj[J_no], F.o2*K[K_b7] + K[K_b6]*x[49]);
    R[51] = -D_r7*x[49] + x[51];
    const T D_r8 = nt_div<T>(K[K_b9]*x[46], K[K_b12]*x[48] + tj[J_no3_no2] + tj[J_no3_no]);
    R[54] = -D_r8*x[48] + x[54];
    const T D_r5 = nt_div<T>(D_r8*tj[J_no3_no] + K[K_b3]*x[45] + tj[J_no2], K[K_a26]*x[47] + K[K_b4]*x[46] + K[K_c5]*x[28] + K[K_d4]*x[52] + K[K_e4]*x[53]);
    R[48] = nt_div<T>(-x[20], D_r5*D_r7 + D_r5 + D_r8 + T(1)) + x[48];
    R[49] = -D_r5*x[48] + x[49];
    const T D_r6 = nt_div<T>(D_r4*F.o2*K[K_a1] + K[K_a30]*x[16] + K[K_a6]*x[46] + K[K_c8]*x[27] + K[K_d8]*x[52] + K[K_e10]*x[53], K[K_a17]*x[43] + K[K_a26]*x[49] + T(2)*K[K_a27]*x[47] + K[K_a6b]*x[46] + K[K_a7]*x[45] + K[K_d10]*x[44] + K[K_d33]*x[52] + K[K_d7]*x[44] + K[K_e15]*x[53] + K[K_e7]*x[50] + T(8.049999999999999e-11)*x[55]);
    R[47] = -D_r6*x[43] + x[47];
    const T D_r13 = nt_div<T>(K[K_d31]*x[48], K[K_d32]*x[45] + het[0]*x[2] + het[1]*x[12] + tj[J_clono2_cl] + tj[J_clono2_clo]);
    const T D_r9 = nt_div<T>(D_r13*het[0]*x[2] + K[K_d33]*x[47], K[K_d35]*x[45] + het[4]*x[12] + tj[J_hocl]);
    const T D_r10 = nt_div<T>(K[K_d60]*x[52], F.hnm*K[K_d61] + tj[J_cl2o2]);
    const T D_r12 = nt_div<T>(K[K_e5c]*x[53], tj[J_brcl]);
    const T D_r11 = nt_div<T>(T(2)*D_r10*tj[J_cl2o2] + D_r12*tj[J_brcl] + D_r13*tj[J_clono2_cl] + D_r9*tj[J_hocl] + K[K_c18]*x[28] + K[K_d3]*x[45] + K[K_d4]*x[49] + K[K_d8]*x[43] + K[K_e5b]*x[53], K[K_d10]*x[47] + K[K_d2]*x[46] + K[K_d37]*x[14] + K[K_d5]*x[1] + K[K_d7]*x[47]);
    R[44] = -D_r11*x[52] + x[44];
    R[52] = nt_div<T>(-x[22], D_r11 + T(1)) + x[52];
    const T D_r27 = nt_div<T>(K[K_e13]*x[48], K[K_e8]*x[45] + tj[J_brono2]);
    const T D_r28 = nt_div<T>(K[K_e15]*x[47], K[K_e16]*x[45] + tj[J_hobr]);
    const T D_r29 = nt_div<T>(K[K_e5c]*x[52], tj[J_brcl]);
    const T D_r30 = nt_div<T>(T(0.85)*D_r27*tj[J_brono2] + D_r28*tj[J_hobr] + D_r29*tj[J_brcl] + K[K_e10]*x[43] + K[K_e3]*x[45] + K[K_e4]*x[49] + K[K_e5a]*x[52] + K[K_e5b]*x[52] + T(2)*K[K_e6]*x[53] + tj[J_bro], K[K_c19]*x[27] + K[K_e2]*x[46] + K[K_e7]*x[47]);
    R[50] = -D_r30*x[53] + x[50];
    R[53] = nt_div<T>(-x[23], D_r30 + T(1)) + x[53];
    const T D_coea = D_r6*(T(1.7e-11)*D_r4 + T(2)*D_r6*K[K_a27] + T(2)*K[K_a17]) + T(2)*K[K_a31];
    const T D_coeb = D_r6*K[K_b23]*x[48] + D_r6*K[K_c7]*x[28] + D_r6*K[K_d33]*x[52] + D_r6*K[K_d7]*x[44] + D_r6*K[K_e15]*x[53] + D_r6*K[K_e7]*x[50] + F.parthbr*K[K_e11]*x[18] + F.parthcl*K[K_d11]*x[12] + F.parthno3*K[K_b27]*x[4] + K[K_b22]*x[48] + K[K_b28]*x[21] + K[K_c17a]*x[29] + K[K_c2]*x[1] + K[K_c8]*x[27] + K[K_d34]*x[14] + K[K_d9]*x[52];
    const T D_coec = D_ch3o*F.o2*K[K_c15] + D_hco*F.o2*K[K_c12] + F.h2*K[K_d6]*x[44] + F.parth2o*x[2]*(T(2)*K[K_a1et]*x[42] + T(2)*tj[J_h2o]) + F.parthno3*tj[J_hno3]*x[4] + K[K_c3]*x[45]*x[56] + K[K_e16]*x[25]*x[45] + tj[J_ch3o2h]*x[29] + T(2)*tj[J_h2o2]*x[16] + tj[J_hbr]*x[18] + tj[J_hobr]*x[25] + x[14]*(K[K_d35]*x[45] + K[K_d37]*x[44] + tj[J_hocl]) + x[21]*(F.hnm*K[K_b24] + tj[J_hno4]) + x[27]*(K[K_c9]*x[45] + tj[J_ch2o_hco]) + x[42]*(T(2.4e-10)*F.h2 + x[1]*(K[K_c1a] + K[K_c1b]));
    const T D_argum_c0 = T(4)*D_coea*D_coec + (D_coeb*D_coeb);
    const bool sel_D_argum = (D_argum_c0) >= (T(0));
    const T D_argum = sel_D_argum ? T(D_argum_c0) : T(T(0));
    R[43] = x[43] + nt_div<T>(-(sqrt(D_argum) - D_coeb), T(2)*D_coea);
    const T D_t06_c0 = tj[J_hocl]*x[14];
    const T D_t06_c1 = K[K_d33]*x[47]*x[52];
    const bool sel_D_t06 = (D_t06_c0) <= (D_t06_c1);
    const T D_t06 = sel_D_t06 ? T(D_t06_c0) : T(D_t06_c1);
    const T D_t07_c0 = K[K_e5c]*x[52]*x[53];
    const T D_t07_c1 = tj[J_brcl]*x[26];
    const bool sel_D_t07 = (D_t07_c0) <= (D_t07_c1);
    const T D_t07 = sel_D_t07 ? T(D_t07_c0) : T(D_t07_c1);
    const T D_t09_c0 = K[K_e15]*x[47]*x[53];
    const T D_t09_c1 = tj[J_hobr]*x[25];
    const bool sel_D_t09 = (D_t09_c0) <= (D_t09_c1);
    const T D_t09 = sel_D_t09 ? T(D_t09_c0) : T(D_t09_c1);
    const T dr7_c0 = T(2)*x[45];
    const T dr7_c1 = nt_div<T>(T(2)*tj[J_no3_no], fmax(T(1e-30), tj[J_no3_no2] + tj[J_no3_no]));
    R[7] = -F.dt*(T(2)*F.o2*tj[J_o2] + K[K_a26]*x[47]*x[49] + K[K_c5]*x[28]*x[49]) + F.dt*(D_t06 + T(2)*D_t07 + D_t09 + K[K_b3]*dr7_c0*x[48] + K[K_b9]*dr7_c1*x[46]*x[48] + K[K_d3]*dr7_c0*x[52] + nt_div<T>(T(2)*K[K_d60]*tj[J_cl2o2]*(x[52]*x[52]), F.hnm*K[K_d61] + tj[J_cl2o2]) + T(2)*K[K_e5b]*x[52]*x[53] + T(2)*K[K_e6]*(x[53]*x[53]) + T(2)*K[K_hk1]*(x[45]*x[45]) + K[K_hk3]*dr7_c0*x[46] + dr7_c1*tj[J_clono2_cl]*x[13] + x[45]*(K[K_a5]*x[43] + K[K_a7]*x[47]) + x[46]*(K[K_a2]*x[55] + K[K_a6]*x[43] + K[K_a6b]*x[47])) - ck0[7] + x[7];
}

// scaled Jacobian J'_ij = dR_i/dx_j s_j / s_i, day equations, into the
// stored A slots (T = double or float; x: FP64 iterate; s: nt_exp_hi scales)
template <typename T, typename FF, typename PK, typename PJ>
__device__ __forceinline__ void nt_jacobian_day(const FF& F, PK K, PK tj, PK het, const double* __restrict__ x, double floor_, PJ J) {
    const int fh = nt_exp_hi(floor_);
    // the iterate in T and the column scales, once per call
    const T xt0 = nt_cvt<T>(x[0]);
    const T xt1 = nt_cvt<T>(x[1]);
    const T xt2 = nt_cvt<T>(x[2]);
    const T xt3 = nt_cvt<T>(x[3]);
    const T xt4 = nt_cvt<T>(x[4]);
    const T xt5 = nt_cvt<T>(x[5]);
    const T xt6 = nt_cvt<T>(x[6]);
    const T xt7 = nt_cvt<T>(x[7]);
    const T xt8 = nt_cvt<T>(x[8]);
    const T xt9 = nt_cvt<T>(x[9]);
    const T xt10 = nt_cvt<T>(x[10]);
    const T xt11 = nt_cvt<T>(x[11]);
    const T xt12 = nt_cvt<T>(x[12]);
    const T xt13 = nt_cvt<T>(x[13]);
    const T xt14 = nt_cvt<T>(x[14]);
    const T xt15 = nt_cvt<T>(x[15]);
    const T xt16 = nt_cvt<T>(x[16]);
    const T xt17 = nt_cvt<T>(x[17]);
    const T xt18 = nt_cvt<T>(x[18]);
    const T xt19 = nt_cvt<T>(x[19]);
    const T xt20 = nt_cvt<T>(x[20]);
    const T xt21 = nt_cvt<T>(x[21]);
    const T xt22 = nt_cvt<T>(x[22]);
    const T xt23 = nt_cvt<T>(x[23]);
    const T xt24 = nt_cvt<T>(x[24]);
    const T xt25 = nt_cvt<T>(x[25]);
    const T xt26 = nt_cvt<T>(x[26]);
    const T xt27 = nt_cvt<T>(x[27]);
    const T xt28 = nt_cvt<T>(x[28]);
    const T xt29 = nt_cvt<T>(x[29]);
    const T xt30 = nt_cvt<T>(x[30]);
    const T xt31 = nt_cvt<T>(x[31]);
    const T xt32 = nt_cvt<T>(x[32]);
    const T xt33 = nt_cvt<T>(x[33]);
    const T xt34 = nt_cvt<T>(x[34]);
    const T xt35 = nt_cvt<T>(x[35]);
    const T xt36 = nt_cvt<T>(x[36]);
    const T xt37 = nt_cvt<T>(x[37]);
    const T xt38 = nt_cvt<T>(x[38]);
    const T xt39 = nt_cvt<T>(x[39]);
    const T xt40 = nt_cvt<T>(x[40]);
    const T xt41 = nt_cvt<T>(x[41]);
    const T xt42 = nt_cvt<T>(x[42]);
    const T xt43 = nt_cvt<T>(x[43]);
    const T xt44 = nt_cvt<T>(x[44]);
    const T xt45 = nt_cvt<T>(x[45]);
    const T xt46 = nt_cvt<T>(x[46]);
    const T xt47 = nt_cvt<T>(x[47]);
    const T xt48 = nt_cvt<T>(x[48]);
    const T xt49 = nt_cvt<T>(x[49]);
    const T xt50 = nt_cvt<T>(x[50]);
    const T xt51 = nt_cvt<T>(x[51]);
    const T xt52 = nt_cvt<T>(x[52]);
    const T xt53 = nt_cvt<T>(x[53]);
    const T xt54 = nt_cvt<T>(x[54]);
    const T xt55 = nt_cvt<T>(x[55]);
    const T xt56 = nt_cvt<T>(x[56]);
    const T cs0 = nt_scale<T>(nt_exp_hi(x[0]), fh);
    const T cs1 = nt_scale<T>(nt_exp_hi(x[1]), fh);
    const T cs2 = nt_scale<T>(nt_exp_hi(x[2]), fh);
    const T cs3 = nt_scale<T>(nt_exp_hi(x[3]), fh);
    const T cs4 = nt_scale<T>(nt_exp_hi(x[4]), fh);
    const T cs5 = nt_scale<T>(nt_exp_hi(x[5]), fh);
    const T cs6 = nt_scale<T>(nt_exp_hi(x[6]), fh);
    const T cs7 = nt_scale<T>(nt_exp_hi(x[7]), fh);
    const T cs8 = nt_scale<T>(nt_exp_hi(x[8]), fh);
    const T cs9 = nt_scale<T>(nt_exp_hi(x[9]), fh);
    const T cs10 = nt_scale<T>(nt_exp_hi(x[10]), fh);
    const T cs11 = nt_scale<T>(nt_exp_hi(x[11]), fh);
    const T cs12 = nt_scale<T>(nt_exp_hi(x[12]), fh);
    const T cs13 = nt_scale<T>(nt_exp_hi(x[13]), fh);
    const T cs14 = nt_scale<T>(nt_exp_hi(x[14]), fh);
    const T cs15 = nt_scale<T>(nt_exp_hi(x[15]), fh);
    const T cs16 = nt_scale<T>(nt_exp_hi(x[16]), fh);
    const T cs17 = nt_scale<T>(nt_exp_hi(x[17]), fh);
    const T cs18 = nt_scale<T>(nt_exp_hi(x[18]), fh);
    const T cs19 = nt_scale<T>(nt_exp_hi(x[19]), fh);
    const T cs20 = nt_scale<T>(nt_exp_hi(x[20]), fh);
    const T cs21 = nt_scale<T>(nt_exp_hi(x[21]), fh);
    const T cs22 = nt_scale<T>(nt_exp_hi(x[22]), fh);
    const T cs23 = nt_scale<T>(nt_exp_hi(x[23]), fh);
    const T cs24 = nt_scale<T>(nt_exp_hi(x[24]), fh);
    const T cs25 = nt_scale<T>(nt_exp_hi(x[25]), fh);
    const T cs26 = nt_scale<T>(nt_exp_hi(x[26]), fh);
    const T cs27 = nt_scale<T>(nt_exp_hi(x[27]), fh);
    const T cs28 = nt_scale<T>(nt_exp_hi(x[28]), fh);
    const T cs29 = nt_scale<T>(nt_exp_hi(x[29]), fh);
    const T cs30 = nt_scale<T>(nt_exp_hi(x[30]), fh);
    const T cs31 = nt_scale<T>(nt_exp_hi(x[31]), fh);
    const T cs32 = nt_scale<T>(nt_exp_hi(x[32]), fh);
    const T cs33 = nt_scale<T>(nt_exp_hi(x[33]), fh);
    const T cs34 = nt_scale<T>(nt_exp_hi(x[34]), fh);
    const T cs35 = nt_scale<T>(nt_exp_hi(x[35]), fh);
    const T cs36 = nt_scale<T>(nt_exp_hi(x[36]), fh);
    const T cs37 = nt_scale<T>(nt_exp_hi(x[37]), fh);
    const T cs38 = nt_scale<T>(nt_exp_hi(x[38]), fh);
    const T cs39 = nt_scale<T>(nt_exp_hi(x[39]), fh);
    const T cs40 = nt_scale<T>(nt_exp_hi(x[40]), fh);
    const T cs41 = nt_scale<T>(nt_exp_hi(x[41]), fh);
    const T cs42 = nt_scale<T>(nt_exp_hi(x[42]), fh);
    const T cs43 = nt_scale<T>(nt_exp_hi(x[43]), fh);
    const T cs44 = nt_scale<T>(nt_exp_hi(x[44]), fh);
    const T cs45 = nt_scale<T>(nt_exp_hi(x[45]), fh);
    const T cs46 = nt_scale<T>(nt_exp_hi(x[46]), fh);
    const T cs47 = nt_scale<T>(nt_exp_hi(x[47]), fh);
    const T cs48 = nt_scale<T>(nt_exp_hi(x[48]), fh);
    const T cs49 = nt_scale<T>(nt_exp_hi(x[49]), fh);
    const T cs50 = nt_scale<T>(nt_exp_hi(x[50]), fh);
    const T cs51 = nt_scale<T>(nt_exp_hi(x[51]), fh);
    const T cs52 = nt_scale<T>(nt_exp_hi(x[52]), fh);
    const T cs53 = nt_scale<T>(nt_exp_hi(x[53]), fh);
    const T cs54 = nt_scale<T>(nt_exp_hi(x[54]), fh);
    const T cs55 = nt_scale<T>(nt_exp_hi(x[55]), fh);
    const T cs56 = nt_scale<T>(nt_exp_hi(x[56]), fh);
    {  // row 0
    const T rs0 = nt_rscale<T>(nt_exp_hi(x[0]), fh);
        const T dj0_c0 = K[K_b38] + K[K_b39];
        J[76] = (F.dt*(dj0_c0*xt42 + tj[J_n2o]) + T(1)) * (cs0 * rs0);
        J[77] = (F.dt*dj0_c0*xt0) * (cs42 * rs0);
    }
    {  // row 1
    const T rs1 = nt_rscale<T>(nt_exp_hi(x[1]), fh);
        const T dj1_c0 = F.dt*xt1;
        J[157] = (F.dt*(K[K_c1a]*xt42 + K[K_c1b]*xt42 + K[K_c1c]*xt42 + K[K_c2]*xt43 + K[K_d5]*xt44) + T(1)) * (cs1 * rs1);
        J[156] = (dj1_c0*(K[K_c1a] + K[K_c1b] + K[K_c1c])) * (cs42 * rs1);
        J[159] = (K[K_c2]*dj1_c0) * (cs43 * rs1);
        J[158] = (K[K_d5]*dj1_c0) * (cs44 * rs1);
    }
    {  // row 2
    const T rs2 = nt_rscale<T>(nt_exp_hi(x[2]), fh);
        const T dj2_c0 = F.dt*xt43;
        const T dj2_c1 = F.dt*F.parth2o;
        const T dj2_c2 = F.parthno3*K[K_b27];
        const T dj2_c3 = F.parthcl*K[K_d11];
        J[261] = (-K[K_c2]*dj2_c0) * (cs1 * rs2);
        J[266] = (dj2_c1*(K[K_a1et]*xt42 + tj[J_h2o]) + T(1)) * (cs2 * rs2);
        J[260] = (-dj2_c0*dj2_c2) * (cs4 * rs2);
        J[265] = (-dj2_c0*dj2_c3) * (cs12 * rs2);
        J[262] = (-K[K_a30]*dj2_c0) * (cs16 * rs2);
        J[264] = (-K[K_c8]*dj2_c0) * (cs27 * rs2);
        J[258] = (-F.dt*(K[K_c17a]*xt43 + K[K_c17b]*xt43)) * (cs29 * rs2);
        J[259] = (K[K_a1et]*dj2_c1*xt2) * (cs42 * rs2);
        J[267] = (-F.dt*(F.h2*K[K_a19] + K[K_a17]*xt47 + K[K_a30]*xt16 + T(2)*K[K_a31]*xt43 + K[K_c17a]*xt29 + K[K_c17b]*xt29 + K[K_c2]*xt1 + K[K_c8]*xt27 + dj2_c2*xt4 + dj2_c3*xt12)) * (cs43 * rs2);
        J[268] = (-F.dt*(K[K_a17]*xt43 + T(1.6e-12)*xt55)) * (cs47 * rs2);
        J[263] = (-T(1.6e-12)*F.dt*xt47) * (cs55 * rs2);
    }
    {  // row 3
    const T rs3 = nt_rscale<T>(nt_exp_hi(x[3]), fh);
        const T dj3_c0 = T(2)*F.dt;
        const T dj3_c1 = K[K_b39]*dj3_c0;
        const T dj3_c2 = K[K_b6]*dj3_c0;
        J[20] = (-dj3_c1*xt42) * (cs0 * rs3);
        J[23] = (F.dt*F.rain_hno3) * (cs4 * rs3);
        J[22] = (-dj3_c1*xt0) * (cs42 * rs3);
        J[24] = (dj3_c2*xt51) * (cs49 * rs3);
        J[21] = (dj3_c2*xt49) * (cs51 * rs3);
    }
    {  // row 4
    const T rs4 = nt_rscale<T>(nt_exp_hi(x[4]), fh);
        const T dj4_c0 = T(2)*het[2];
        const T dj4_c1 = F.dt*K[K_b22];
        J[122] = (-F.dt*(dj4_c0*xt5 + het[0]*xt13 + het[5]*xt19)) * (cs2 * rs4);
        J[120] = (F.dt*(F.parthno3*(K[K_b27]*xt43 + tj[J_hno3]) + F.rain_hno3) + T(1)) * (cs4 * rs4);
        J[118] = (-F.dt*(dj4_c0*xt2 + het[3]*xt12)) * (cs5 * rs4);
        J[121] = (-F.dt*(het[1]*xt13 + het[3]*xt5)) * (cs12 * rs4);
        J[119] = (-F.dt*(het[0]*xt2 + het[1]*xt12)) * (cs13 * rs4);
        J[117] = (-F.dt*het[5]*xt2) * (cs19 * rs4);
        J[124] = (F.dt*F.parthno3*K[K_b27]*xt4 - dj4_c1*xt48) * (cs43 * rs4);
        J[123] = (-dj4_c1*xt43) * (cs48 * rs4);
    }
    {  // row 5
    const T rs5 = nt_rscale<T>(nt_exp_hi(x[5]), fh);
        const T dj5_c0 = F.dt*xt5;
        const T dj5_c1 = F.dt*K[K_b12];
        J[74] = (dj5_c0*het[2]) * (cs2 * rs5);
        J[72] = (F.dt*(F.hnm*K[K_b32] + het[2]*xt2 + het[3]*xt12 + tj[J_n2o5]) + T(1)) * (cs5 * rs5);
        J[73] = (dj5_c0*het[3]) * (cs12 * rs5);
        J[75] = (-dj5_c1*xt54) * (cs48 * rs5);
        J[71] = (-dj5_c1*xt48) * (cs54 * rs5);
    }
    {  // row 6
    const T rs6 = nt_rscale<T>(nt_exp_hi(x[6]), fh);
        const T dj6_c0 = T(3)*xt42;
        const T dj6_c1 = T(2)*K[K_d91];
        const T dj6_c2 = T(4)*K[K_d93];
        const T dj6_c3 = T(3)*K[K_d94];
        J[9] = (F.dt*F.rain_hcl) * (cs12 * rs6);
        J[7] = (-F.dt*(K[K_d90]*dj6_c0 + T(3)*tj[J_cfc11])) * (cs30 * rs6);
        J[4] = (-F.dt*(dj6_c1*xt42 + T(2)*tj[J_cfc12])) * (cs31 * rs6);
        J[0] = (-F.dt*(K[K_d92]*dj6_c0 + T(3)*tj[J_cfc113])) * (cs32 * rs6);
        J[2] = (-F.dt*(dj6_c2*xt42 + T(4)*tj[J_ccl4])) * (cs33 * rs6);
        J[6] = (-F.dt*(dj6_c3*xt43 + T(3)*tj[J_ch3ccl3])) * (cs34 * rs6);
        J[5] = (-F.dt*(K[K_d95]*xt43 + tj[J_ch3cl])) * (cs35 * rs6);
        J[3] = (-F.dt*(K[K_d96]*xt42 + K[K_d97]*xt43 + tj[J_hcfc22])) * (cs36 * rs6);
        J[1] = (-F.dt*(K[K_e52]*xt42 + tj[J_h1211])) * (cs38 * rs6);
        J[8] = (-F.dt*(T(3)*K[K_d90]*xt30 + T(3)*K[K_d92]*xt32 + K[K_d96]*xt36 + K[K_e52]*xt38 + dj6_c1*xt31 + dj6_c2*xt33)) * (cs42 * rs6);
        J[10] = (-F.dt*(K[K_d95]*xt35 + K[K_d97]*xt36 + dj6_c3*xt34)) * (cs43 * rs6);
    }
    {  // row 9
    const T rs9 = nt_rscale<T>(nt_exp_hi(x[9]), fh);
        const T dj9_c0 = F.dt*K[K_e5a];
        J[100] = (F.dt*tj[J_oclo] + T(1)) * (cs9 * rs9);
        J[102] = (-dj9_c0*xt53) * (cs52 * rs9);
        J[101] = (-dj9_c0*xt52) * (cs53 * rs9);
    }
    {  // row 10
    const T rs10 = nt_rscale<T>(nt_exp_hi(x[10]), fh);
    }
    {  // row 11
    const T rs11 = nt_rscale<T>(nt_exp_hi(x[11]), fh);
    }
    {  // row 12
    const T rs12 = nt_rscale<T>(nt_exp_hi(x[12]), fh);
        const T dj12_c0 = F.dt*xt44;
        const T dj12_c1 = F.dt*xt12;
        const T dj12_c2 = F.dt*K[K_d9];
        J[250] = (-K[K_d5]*dj12_c0) * (cs1 * rs12);
        J[247] = (dj12_c1*het[3]) * (cs5 * rs12);
        J[253] = (F.dt*(F.parthcl*(K[K_d11]*xt43 + tj[J_hcl]) + F.rain_hcl + het[1]*xt13 + het[3]*xt5 + het[4]*xt14 + het[6]*xt25) + T(1)) * (cs12 * rs12);
        J[249] = (dj12_c1*het[1]) * (cs13 * rs12);
        J[251] = (dj12_c1*het[4]) * (cs14 * rs12);
        J[248] = (dj12_c1*het[6]) * (cs25 * rs12);
        J[252] = (-K[K_c10]*dj12_c0) * (cs27 * rs12);
        J[255] = (F.parthcl*K[K_d11]*dj12_c1 - dj12_c2*xt52) * (cs43 * rs12);
        J[254] = (-F.dt*(F.h2*K[K_d6] + K[K_c10]*xt27 + K[K_d5]*xt1 + K[K_d7]*xt47)) * (cs44 * rs12);
        J[256] = (-K[K_d7]*dj12_c0) * (cs47 * rs12);
        J[257] = (-dj12_c2*xt43) * (cs52 * rs12);
    }
    {  // row 13
    const T rs13 = nt_rscale<T>(nt_exp_hi(x[13]), fh);
        const T dj13_c0 = F.dt*xt13;
        const T dj13_c1 = F.dt*K[K_d31];
        J[89] = (dj13_c0*het[0]) * (cs2 * rs13);
        J[88] = (dj13_c0*het[1]) * (cs12 * rs13);
        J[87] = (F.dt*(K[K_d32]*xt45 + het[0]*xt2 + het[1]*xt12 + tj[J_clono2_cl] + tj[J_clono2_clo]) + T(1)) * (cs13 * rs13);
        J[91] = (K[K_d32]*dj13_c0) * (cs45 * rs13);
        J[90] = (-dj13_c1*xt52) * (cs48 * rs13);
        J[92] = (-dj13_c1*xt48) * (cs52 * rs13);
    }
    {  // row 14
    const T rs14 = nt_rscale<T>(nt_exp_hi(x[14]), fh);
        const T dj14_c0 = F.dt*het[0];
        const T dj14_c1 = F.dt*xt14;
        const T dj14_c2 = F.dt*K[K_d33];
        J[170] = (-dj14_c0*xt13) * (cs2 * rs14);
        J[169] = (dj14_c1*het[4]) * (cs12 * rs14);
        J[166] = (-dj14_c0*xt2) * (cs13 * rs14);
        J[167] = (F.dt*(K[K_d34]*xt43 + K[K_d35]*xt45 + K[K_d37]*xt44 + het[4]*xt12 + het[8]*xt18 + tj[J_hocl]) + T(1)) * (cs14 * rs14);
        J[168] = (dj14_c1*het[8]) * (cs18 * rs14);
        J[173] = (K[K_d34]*dj14_c1) * (cs43 * rs14);
        J[172] = (K[K_d37]*dj14_c1) * (cs44 * rs14);
        J[171] = (K[K_d35]*dj14_c1) * (cs45 * rs14);
        J[174] = (-dj14_c2*xt52) * (cs47 * rs14);
        J[175] = (-dj14_c2*xt47) * (cs52 * rs14);
    }
    {  // row 15
    const T rs15 = nt_rscale<T>(nt_exp_hi(x[15]), fh);
        J[63] = (-F.dt*(het[1]*xt13 + het[4]*xt14)) * (cs12 * rs15);
        J[61] = (-F.dt*het[1]*xt12) * (cs13 * rs15);
        J[62] = (-F.dt*(K[K_d37]*xt44 + het[4]*xt12)) * (cs14 * rs15);
        J[60] = (F.dt*tj[J_cl2] + T(1)) * (cs15 * rs15);
        J[64] = (-F.dt*K[K_d37]*xt14) * (cs44 * rs15);
        J[65] = (-T(2)*F.dt*K[K_d62]*xt52) * (cs52 * rs15);
    }
    {  // row 16
    const T rs16 = nt_rscale<T>(nt_exp_hi(x[16]), fh);
        J[189] = (F.dt*(F.rain_h2o2 + K[K_a30]*xt43 + tj[J_h2o2]) + T(1)) * (cs16 * rs16);
        J[190] = (F.dt*K[K_a30]*xt16) * (cs43 * rs16);
        J[191] = (-T(2)*F.dt*K[K_a27]*xt47) * (cs47 * rs16);
    }
    {  // row 17
    const T rs17 = nt_rscale<T>(nt_exp_hi(x[17]), fh);
        const T dj17_c0 = F.dt*het[3];
        const T dj17_c1 = F.dt*K[K_d36];
        J[26] = (-dj17_c0*xt12) * (cs5 * rs17);
        J[27] = (-dj17_c0*xt5) * (cs12 * rs17);
        J[25] = (F.dt*tj[J_clno2] + T(1)) * (cs17 * rs17);
        J[29] = (-dj17_c1*xt48) * (cs44 * rs17);
        J[28] = (-dj17_c1*xt44) * (cs48 * rs17);
    }
    {  // row 18
    const T rs18 = nt_rscale<T>(nt_exp_hi(x[18]), fh);
        const T dj18_c0 = F.dt*xt18;
        const T dj18_c1 = F.dt*xt50;
        const T dj18_c2 = F.parthbr*dj18_c0;
        J[183] = (dj18_c0*het[8]) * (cs14 * rs18);
        J[184] = (F.dt*(F.parthbr*(K[K_e11]*xt43 + K[K_e9]*xt42 + tj[J_hbr]) + F.rain_hbr + het[7]*xt25 + het[8]*xt14) + T(1)) * (cs18 * rs18);
        J[181] = (dj18_c0*het[7]) * (cs25 * rs18);
        J[185] = (-K[K_c19]*dj18_c1) * (cs27 * rs18);
        J[182] = (K[K_e9]*dj18_c2) * (cs42 * rs18);
        J[187] = (K[K_e11]*dj18_c2) * (cs43 * rs18);
        J[188] = (-K[K_e7]*dj18_c1) * (cs47 * rs18);
        J[186] = (-F.dt*(K[K_c19]*xt27 + K[K_e7]*xt47)) * (cs50 * rs18);
    }
    {  // row 19
    const T rs19 = nt_rscale<T>(nt_exp_hi(x[19]), fh);
        const T dj19_c0 = F.dt*xt19;
        const T dj19_c1 = F.dt*K[K_e13];
        J[56] = (dj19_c0*het[5]) * (cs2 * rs19);
        J[55] = (F.dt*(K[K_e8]*xt45 + het[5]*xt2 + tj[J_brono2]) + T(1)) * (cs19 * rs19);
        J[58] = (K[K_e8]*dj19_c0) * (cs45 * rs19);
        J[57] = (-dj19_c1*xt53) * (cs48 * rs19);
        J[59] = (-dj19_c1*xt48) * (cs53 * rs19);
    }
    {  // row 20
    const T rs20 = nt_rscale<T>(nt_exp_hi(x[20]), fh);
        const T dj20_c0 = T(2)*F.dt;
        const T dj20_c1 = K[K_b39]*dj20_c0;
        const T dj20_c2 = F.parthno3*K[K_b27];
        const T dj20_c3 = F.dt*xt48;
        const T dj20_c4 = T(2)*K[K_b12];
        const T dj20_c5 = K[K_b6]*dj20_c0;
        J[233] = (-dj20_c1*xt42) * (cs0 * rs20);
        J[237] = (-F.dt*(F.parthno3*tj[J_hno3] + dj20_c2*xt43)) * (cs4 * rs20);
        J[232] = (-F.dt*(T(2)*F.hnm*K[K_b32] + T(2)*tj[J_n2o5])) * (cs5 * rs20);
        J[235] = (-F.dt*(K[K_d32]*xt45 + tj[J_clono2_cl] + tj[J_clono2_clo])) * (cs13 * rs20);
        J[229] = (-F.dt*tj[J_clno2]) * (cs17 * rs20);
        J[230] = (-F.dt*(K[K_e8]*xt45 + tj[J_brono2])) * (cs19 * rs20);
        J[238] = (-F.dt*(F.hnm*K[K_b24] + K[K_b28]*xt43 + tj[J_hno4])) * (cs21 * rs20);
        J[236] = (-dj20_c1*xt0) * (cs42 * rs20);
        J[243] = (-F.dt*(K[K_b28]*xt21 + dj20_c2*xt4) + K[K_b22]*dj20_c3) * (cs43 * rs20);
        J[241] = (K[K_d36]*dj20_c3) * (cs44 * rs20);
        J[240] = (-F.dt*(K[K_d32]*xt13 + K[K_e8]*xt19)) * (cs45 * rs20);
        J[244] = (K[K_b23]*dj20_c3) * (cs47 * rs20);
        J[239] = (F.dt*(K[K_b22]*xt43 + K[K_b23]*xt47 + K[K_d31]*xt52 + K[K_d36]*xt44 + K[K_e13]*xt53 + dj20_c4*xt54)) * (cs48 * rs20);
        J[245] = (dj20_c5*xt51) * (cs49 * rs20);
        J[234] = (dj20_c5*xt49) * (cs51 * rs20);
        J[246] = (K[K_d31]*dj20_c3) * (cs52 * rs20);
        J[242] = (K[K_e13]*dj20_c3) * (cs53 * rs20);
        J[231] = (dj20_c3*dj20_c4) * (cs54 * rs20);
    }
    {  // row 21
    const T rs21 = nt_rscale<T>(nt_exp_hi(x[21]), fh);
        const T dj21_c0 = F.dt*K[K_b23];
        J[152] = (F.dt*(F.hnm*K[K_b24] + K[K_b28]*xt43 + tj[J_hno4]) + T(1)) * (cs21 * rs21);
        J[154] = (F.dt*K[K_b28]*xt21) * (cs43 * rs21);
        J[155] = (-dj21_c0*xt48) * (cs47 * rs21);
        J[153] = (-dj21_c0*xt47) * (cs48 * rs21);
    }
    {  // row 22
    const T rs22 = nt_rscale<T>(nt_exp_hi(x[22]), fh);
        const T dj22_c0 = F.dt*xt44;
        const T dj22_c1 = T(3)*xt42;
        const T dj22_c2 = T(2)*K[K_d91];
        const T dj22_c3 = T(4)*K[K_d93];
        const T dj22_c4 = T(3)*K[K_d94];
        const T dj22_c5 = F.dt*xt52;
        const T dj22_c6 = T(2)*K[K_d60];
        const T dj22_c7 = T(2)*K[K_d62];
        J[141] = (K[K_d5]*dj22_c0) * (cs1 * rs22);
        J[140] = (-F.dt*tj[J_oclo]) * (cs9 * rs22);
        J[144] = (-F.dt*F.parthcl*(K[K_d11]*xt43 + tj[J_hcl])) * (cs12 * rs22);
        J[135] = (-F.dt*(K[K_d32]*xt45 + tj[J_clono2_cl] + tj[J_clono2_clo])) * (cs13 * rs22);
        J[142] = (-F.dt*(K[K_d34]*xt43 + K[K_d35]*xt45 + tj[J_hocl]) + K[K_d37]*dj22_c0) * (cs14 * rs22);
        J[133] = (-T(2)*F.dt*tj[J_cl2]) * (cs15 * rs22);
        J[128] = (-F.dt*tj[J_clno2]) * (cs17 * rs22);
        J[138] = (-F.dt*(T(2)*F.hnm*K[K_d61] + T(2)*tj[J_cl2o2])) * (cs24 * rs22);
        J[132] = (-F.dt*tj[J_brcl]) * (cs26 * rs22);
        J[143] = (K[K_c10]*dj22_c0) * (cs27 * rs22);
        J[137] = (-F.dt*(K[K_d90]*dj22_c1 + T(3)*tj[J_cfc11])) * (cs30 * rs22);
        J[131] = (-F.dt*(dj22_c2*xt42 + T(2)*tj[J_cfc12])) * (cs31 * rs22);
        J[127] = (-F.dt*(K[K_d92]*dj22_c1 + T(3)*tj[J_cfc113])) * (cs32 * rs22);
        J[129] = (-F.dt*(dj22_c3*xt42 + T(4)*tj[J_ccl4])) * (cs33 * rs22);
        J[136] = (-F.dt*(dj22_c4*xt43 + T(3)*tj[J_ch3ccl3])) * (cs34 * rs22);
        J[134] = (-F.dt*(K[K_d95]*xt43 + tj[J_ch3cl])) * (cs35 * rs22);
        J[130] = (-F.dt*(K[K_d96]*xt42 + K[K_d97]*xt43 + tj[J_hcfc22])) * (cs36 * rs22);
        J[139] = (-F.dt*(T(3)*K[K_d90]*xt30 + T(3)*K[K_d92]*xt32 + K[K_d96]*xt36 + dj22_c2*xt31 + dj22_c3*xt33)) * (cs42 * rs22);
        J[149] = (-F.dt*(F.parthcl*K[K_d11]*xt12 + K[K_d34]*xt14 + K[K_d95]*xt35 + K[K_d97]*xt36 + dj22_c4*xt34) + K[K_d9]*dj22_c5) * (cs43 * rs22);
        J[147] = (F.dt*(F.h2*K[K_d6] + K[K_c10]*xt27 + K[K_d36]*xt48 + K[K_d37]*xt14 + K[K_d5]*xt1 + K[K_d7]*xt47)) * (cs44 * rs22);
        J[146] = (-F.dt*(K[K_d32]*xt13 + K[K_d35]*xt14)) * (cs45 * rs22);
        J[150] = (F.dt*(K[K_d33]*xt52 + K[K_d7]*xt44)) * (cs47 * rs22);
        J[145] = (F.dt*(K[K_d31]*xt52 + K[K_d36]*xt44)) * (cs48 * rs22);
        J[151] = (F.dt*(K[K_d31]*xt48 + K[K_d33]*xt47 + K[K_d9]*xt43 + K[K_e5a]*xt53 + K[K_e5c]*xt53 + dj22_c6*xt52 + dj22_c7*xt52 + xt52*(dj22_c6 + dj22_c7))) * (cs52 * rs22);
        J[148] = (dj22_c5*(K[K_e5a] + K[K_e5c])) * (cs53 * rs22);
    }
    {  // row 23
    const T rs23 = nt_rscale<T>(nt_exp_hi(x[23]), fh);
        const T dj23_c0 = T(2)*het[7];
        const T dj23_c1 = F.dt*F.parthbr*xt18;
        const T dj23_c2 = F.dt*xt53;
        J[196] = (-F.dt*(F.parthbr*(K[K_e11]*xt43 + K[K_e9]*xt42 + tj[J_hbr]) + dj23_c0*xt25)) * (cs18 * rs23);
        J[193] = (-F.dt*(K[K_e8]*xt45 + tj[J_brono2])) * (cs19 * rs23);
        J[194] = (-F.dt*(K[K_e16]*xt45 + dj23_c0*xt18 + tj[J_hobr])) * (cs25 * rs23);
        J[192] = (-F.dt*tj[J_brcl]) * (cs26 * rs23);
        J[197] = (F.dt*K[K_c19]*xt50) * (cs27 * rs23);
        J[195] = (-K[K_e9]*dj23_c1) * (cs42 * rs23);
        J[202] = (-K[K_e11]*dj23_c1) * (cs43 * rs23);
        J[199] = (-F.dt*(K[K_e16]*xt25 + K[K_e8]*xt19)) * (cs45 * rs23);
        J[203] = (F.dt*(K[K_e15]*xt53 + K[K_e7]*xt50)) * (cs47 * rs23);
        J[198] = (K[K_e13]*dj23_c2) * (cs48 * rs23);
        J[201] = (F.dt*(K[K_c19]*xt27 + K[K_e7]*xt47)) * (cs50 * rs23);
        J[204] = (K[K_e5c]*dj23_c2) * (cs52 * rs23);
        J[200] = (F.dt*(K[K_e13]*xt48 + K[K_e15]*xt47 + K[K_e5c]*xt52)) * (cs53 * rs23);
    }
    {  // row 24
    const T rs24 = nt_rscale<T>(nt_exp_hi(x[24]), fh);
        J[97] = (F.dt*(F.hnm*K[K_d61] + tj[J_cl2o2]) + T(1)) * (cs24 * rs24);
        J[98] = (-T(2)*F.dt*K[K_d60]*xt52) * (cs52 * rs24);
    }
    {  // row 25
    const T rs25 = nt_rscale<T>(nt_exp_hi(x[25]), fh);
        const T dj25_c0 = F.dt*het[5];
        const T dj25_c1 = F.dt*xt25;
        const T dj25_c2 = F.dt*K[K_e15];
        J[83] = (-dj25_c0*xt19) * (cs2 * rs25);
        J[82] = (dj25_c1*het[6]) * (cs12 * rs25);
        J[81] = (dj25_c1*het[7]) * (cs18 * rs25);
        J[79] = (-dj25_c0*xt2) * (cs19 * rs25);
        J[80] = (F.dt*(K[K_e16]*xt45 + het[6]*xt12 + het[7]*xt18 + tj[J_hobr]) + T(1)) * (cs25 * rs25);
        J[84] = (K[K_e16]*dj25_c1) * (cs45 * rs25);
        J[86] = (-dj25_c2*xt53) * (cs47 * rs25);
        J[85] = (-dj25_c2*xt47) * (cs53 * rs25);
    }
    {  // row 26
    const T rs26 = nt_rscale<T>(nt_exp_hi(x[26]), fh);
        const T dj26_c0 = F.dt*het[6];
        const T dj26_c1 = F.dt*het[8];
        const T dj26_c2 = F.dt*K[K_e5c];
        J[47] = (-dj26_c0*xt25) * (cs12 * rs26);
        J[45] = (-dj26_c1*xt18) * (cs14 * rs26);
        J[46] = (-dj26_c1*xt14) * (cs18 * rs26);
        J[44] = (-dj26_c0*xt12) * (cs25 * rs26);
        J[43] = (F.dt*tj[J_brcl] + T(1)) * (cs26 * rs26);
        J[49] = (-dj26_c2*xt53) * (cs52 * rs26);
        J[48] = (-dj26_c2*xt52) * (cs53 * rs26);
    }
    {  // row 28
    const T rs28 = nt_rscale<T>(nt_exp_hi(x[28]), fh);
        const T dj28_c0 = T(2)*K[K_c14]*xt28;
        const T dj28_c1 = F.dt*K[K_c17a];
        const T dj28_c2 = F.dt*xt28;
        J[212] = (F.dt*dj28_c0 + F.dt*(K[K_c18]*xt52 + K[K_c5]*xt49 + K[K_c7]*xt47 + dj28_c0) + T(1)) * (cs28 * rs28);
        J[210] = (-dj28_c1*xt43) * (cs29 * rs28);
        J[213] = (-dj28_c1*xt29) * (cs43 * rs28);
        J[214] = (K[K_c7]*dj28_c2) * (cs47 * rs28);
        J[215] = (K[K_c5]*dj28_c2) * (cs49 * rs28);
        J[216] = (K[K_c18]*dj28_c2) * (cs52 * rs28);
        J[211] = (-F.dt*F.o2*K[K_c4]) * (cs56 * rs28);
    }
    {  // row 29
    const T rs29 = nt_rscale<T>(nt_exp_hi(x[29]), fh);
        const T dj29_c0 = F.dt*K[K_c7];
        J[35] = (-dj29_c0*xt47) * (cs28 * rs29);
        J[34] = (F.dt*(K[K_c17a]*xt43 + K[K_c17b]*xt43 + tj[J_ch3o2h]) + T(1)) * (cs29 * rs29);
        J[36] = (F.dt*xt29*(K[K_c17a] + K[K_c17b])) * (cs43 * rs29);
        J[37] = (-dj29_c0*xt28) * (cs47 * rs29);
    }
    {  // row 30
    const T rs30 = nt_rscale<T>(nt_exp_hi(x[30]), fh);
        J[95] = (F.dt*(K[K_d90]*xt42 + tj[J_cfc11]) + T(1)) * (cs30 * rs30);
        J[96] = (F.dt*K[K_d90]*xt30) * (cs42 * rs30);
    }
    {  // row 31
    const T rs31 = nt_rscale<T>(nt_exp_hi(x[31]), fh);
        J[41] = (F.dt*(K[K_d91]*xt42 + tj[J_cfc12]) + T(1)) * (cs31 * rs31);
        J[42] = (F.dt*K[K_d91]*xt31) * (cs42 * rs31);
    }
    {  // row 32
    const T rs32 = nt_rscale<T>(nt_exp_hi(x[32]), fh);
        J[18] = (F.dt*(K[K_d92]*xt42 + tj[J_cfc113]) + T(1)) * (cs32 * rs32);
        J[19] = (F.dt*K[K_d92]*xt32) * (cs42 * rs32);
    }
    {  // row 33
    const T rs33 = nt_rscale<T>(nt_exp_hi(x[33]), fh);
        J[32] = (F.dt*(K[K_d93]*xt42 + tj[J_ccl4]) + T(1)) * (cs33 * rs33);
        J[33] = (F.dt*K[K_d93]*xt33) * (cs42 * rs33);
    }
    {  // row 34
    const T rs34 = nt_rscale<T>(nt_exp_hi(x[34]), fh);
        J[93] = (F.dt*(K[K_d94]*xt43 + tj[J_ch3ccl3]) + T(1)) * (cs34 * rs34);
        J[94] = (F.dt*K[K_d94]*xt34) * (cs43 * rs34);
    }
    {  // row 35
    const T rs35 = nt_rscale<T>(nt_exp_hi(x[35]), fh);
        J[66] = (F.dt*(K[K_d95]*xt43 + tj[J_ch3cl]) + T(1)) * (cs35 * rs35);
        J[67] = (F.dt*K[K_d95]*xt35) * (cs43 * rs35);
    }
    {  // row 36
    const T rs36 = nt_rscale<T>(nt_exp_hi(x[36]), fh);
        const T dj36_c0 = F.dt*xt36;
        J[38] = (F.dt*(K[K_d96]*xt42 + K[K_d97]*xt43 + tj[J_hcfc22]) + T(1)) * (cs36 * rs36);
        J[39] = (K[K_d96]*dj36_c0) * (cs42 * rs36);
        J[40] = (K[K_d97]*dj36_c0) * (cs43 * rs36);
    }
    {  // row 37
    const T rs37 = nt_rscale<T>(nt_exp_hi(x[37]), fh);
        const T dj37_c0 = F.dt*xt37;
        J[52] = (F.dt*(K[K_e50]*xt42 + K[K_e51]*xt43 + tj[J_ch3br]) + T(1)) * (cs37 * rs37);
        J[53] = (K[K_e50]*dj37_c0) * (cs42 * rs37);
        J[54] = (K[K_e51]*dj37_c0) * (cs43 * rs37);
    }
    {  // row 38
    const T rs38 = nt_rscale<T>(nt_exp_hi(x[38]), fh);
        J[30] = (F.dt*(K[K_e52]*xt42 + tj[J_h1211]) + T(1)) * (cs38 * rs38);
        J[31] = (F.dt*K[K_e52]*xt38) * (cs42 * rs38);
    }
    {  // row 39
    const T rs39 = nt_rscale<T>(nt_exp_hi(x[39]), fh);
        J[50] = (F.dt*(K[K_e53]*xt42 + tj[J_h1301]) + T(1)) * (cs39 * rs39);
        J[51] = (F.dt*K[K_e53]*xt39) * (cs42 * rs39);
    }
    {  // row 40
    const T rs40 = nt_rscale<T>(nt_exp_hi(x[40]), fh);
        const T dj40_c0 = T(2)*K[K_e54];
        J[16] = (F.dt*F.rain_hbr) * (cs18 * rs40);
        J[13] = (-F.dt*(K[K_e50]*xt42 + K[K_e51]*xt43 + tj[J_ch3br])) * (cs37 * rs40);
        J[11] = (-F.dt*(K[K_e52]*xt42 + tj[J_h1211])) * (cs38 * rs40);
        J[12] = (-F.dt*(K[K_e53]*xt42 + tj[J_h1301])) * (cs39 * rs40);
        J[15] = (-F.dt*(dj40_c0*xt43 + T(2)*tj[J_ch2br2])) * (cs41 * rs40);
        J[14] = (-F.dt*(K[K_e50]*xt37 + K[K_e52]*xt38 + K[K_e53]*xt39)) * (cs42 * rs40);
        J[17] = (-F.dt*(K[K_e51]*xt37 + dj40_c0*xt41)) * (cs43 * rs40);
    }
    {  // row 41
    const T rs41 = nt_rscale<T>(nt_exp_hi(x[41]), fh);
        J[125] = (F.dt*(K[K_e54]*xt43 + tj[J_ch2br2]) + T(1)) * (cs41 * rs41);
        J[126] = (F.dt*K[K_e54]*xt41) * (cs43 * rs41);
    }
    {  // row 42
    const T rs42 = nt_rscale<T>(nt_exp_hi(x[42]), fh);
        J[99] = (nt_div<T>(-tj[J_o3_o1d], F.n2*K[K_hk4] + F.o2*K[K_hk5])) * (cs46 * rs42);
    }
    {  // row 56
    const T rs56 = nt_rscale<T>(nt_exp_hi(x[56]), fh);
        const T dj56_c0 = F.o2*K[K_c4] + K[K_c3]*xt45;
        const T dj56_c1 = nt_div<T>(T(1), dj56_c0);
        const T dj56_c2 = K[K_c1a]*xt42 + K[K_c2]*xt43 + K[K_d5]*xt44;
        const T dj56_c3 = dj56_c1*xt1;
        J[177] = (-dj56_c1*dj56_c2) * (cs1 * rs56);
        J[176] = (-K[K_c1a]*dj56_c3) * (cs42 * rs56);
        J[180] = (-K[K_c2]*dj56_c3) * (cs43 * rs56);
        J[179] = (-K[K_d5]*dj56_c3) * (cs44 * rs56);
        J[178] = (nt_div<T>(K[K_c3]*dj56_c2*xt1, (dj56_c0*dj56_c0))) * (cs45 * rs56);
    }
    const T D_ch3o_c0 = K[K_c1b]*xt42;
    const T D_ch3o_c1 = K[K_c14]*xt28;
    const T D_ch3o_c2 = K[K_c18]*xt52 + K[K_c5]*xt49;
    const T D_ch3o_c3 = nt_div<T>(T(1), F.o2*K[K_c15]);
    const T D_ch3o_c4 = D_ch3o_c3*xt28;
    const T D_ch3o = D_ch3o_c3*(D_ch3o_c0*xt1 + tj[J_ch3o2h]*xt29 + xt28*(T(2)*D_ch3o_c1 + D_ch3o_c2));
    const T d_D_ch3o_1 = D_ch3o_c0*D_ch3o_c3;
    const T d_D_ch3o_28 = D_ch3o_c3*(T(4)*D_ch3o_c1 + D_ch3o_c2);
    const T d_D_ch3o_29 = D_ch3o_c3*tj[J_ch3o2h];
    const T d_D_ch3o_42 = D_ch3o_c3*K[K_c1b]*xt1;
    const T d_D_ch3o_49 = D_ch3o_c4*K[K_c5];
    const T d_D_ch3o_52 = D_ch3o_c4*K[K_c18];
    {  // row 27
    const T rs27 = nt_rscale<T>(nt_exp_hi(x[27]), fh);
        const T dj27_c0 = F.dt*K[K_c1c];
        const T dj27_c1 = F.dt*F.o2*K[K_c15];
        const T dj27_c2 = F.dt*K[K_c17b];
        const T dj27_c3 = F.dt*xt27;
        const T dj27_c4 = F.dt*K[K_c3];
        J[219] = (-d_D_ch3o_1*dj27_c1 - dj27_c0*xt42) * (cs1 * rs27);
        J[222] = (F.dt*(K[K_c10]*xt44 + K[K_c19]*xt50 + K[K_c8]*xt43 + K[K_c9]*xt45 + tj[J_ch2o_co] + tj[J_ch2o_hco]) + T(1)) * (cs27 * rs27);
        J[221] = (-d_D_ch3o_28*dj27_c1) * (cs28 * rs27);
        J[217] = (-d_D_ch3o_29*dj27_c1 - dj27_c2*xt43) * (cs29 * rs27);
        J[218] = (-d_D_ch3o_42*dj27_c1 - dj27_c0*xt1) * (cs42 * rs27);
        J[226] = (F.dt*K[K_c8]*xt27 - dj27_c2*xt29) * (cs43 * rs27);
        J[224] = (K[K_c10]*dj27_c3) * (cs44 * rs27);
        J[223] = (F.dt*K[K_c9]*xt27 - dj27_c4*xt56) * (cs45 * rs27);
        J[227] = (-d_D_ch3o_49*dj27_c1) * (cs49 * rs27);
        J[225] = (K[K_c19]*dj27_c3) * (cs50 * rs27);
        J[228] = (-d_D_ch3o_52*dj27_c1) * (cs52 * rs27);
        J[220] = (-dj27_c4*xt45) * (cs56 * rs27);
    }
    const T D_hco_c0 = nt_div<T>(T(1), F.o2*K[K_c12]);
    const T D_hco_c1 = D_hco_c0*(K[K_c10]*xt44 + K[K_c19]*xt50 + K[K_c8]*xt43 + K[K_c9]*xt45 + tj[J_ch2o_hco]);
    const T D_hco_c2 = D_hco_c0*xt27;
    const T D_hco = D_hco_c1*xt27;
    const T d_D_hco_27 = D_hco_c1;
    const T d_D_hco_43 = D_hco_c2*K[K_c8];
    const T d_D_hco_44 = D_hco_c2*K[K_c10];
    const T d_D_hco_45 = D_hco_c2*K[K_c9];
    const T d_D_hco_50 = D_hco_c2*K[K_c19];
    {  // row 8
    const T rs8 = nt_rscale<T>(nt_exp_hi(x[8]), fh);
        const T dj8_c0 = F.dt*F.o2*K[K_c12];
        J[160] = (F.dt*K[K_a36]*xt43 + T(1)) * (cs8 * rs8);
        J[161] = (-F.dt*tj[J_ch2o_co] - d_D_hco_27*dj8_c0) * (cs27 * rs8);
        J[165] = (F.dt*K[K_a36]*xt8 - d_D_hco_43*dj8_c0) * (cs43 * rs8);
        J[163] = (-d_D_hco_44*dj8_c0) * (cs44 * rs8);
        J[162] = (-d_D_hco_45*dj8_c0) * (cs45 * rs8);
        J[164] = (-d_D_hco_50*dj8_c0) * (cs50 * rs8);
    }
    const T D_r1_c0 = nt_div<T>(T(1), F.o2*K[K_hk2]);
    const T D_r1 = D_r1_c0*(K[K_a2]*xt55 + K[K_a6]*xt43 + K[K_a6b]*xt47 + K[K_b4]*xt49 + K[K_d2]*xt44 + tj[J_o3_o1d] + tj[J_o3_o3p]);
    const T d_D_r1_43 = D_r1_c0*K[K_a6];
    const T d_D_r1_44 = D_r1_c0*K[K_d2];
    const T d_D_r1_47 = D_r1_c0*K[K_a6b];
    const T d_D_r1_49 = D_r1_c0*K[K_b4];
    const T d_D_r1_55 = D_r1_c0*K[K_a2];
    {  // row 45
    const T rs45 = nt_rscale<T>(nt_exp_hi(x[45]), fh);
        J[280] = (-d_D_r1_43*xt46) * (cs43 * rs45);
        J[279] = (-d_D_r1_44*xt46) * (cs44 * rs45);
        J[282] = (-D_r1) * (cs46 * rs45);
        J[281] = (-d_D_r1_47*xt46) * (cs47 * rs45);
        J[283] = (-d_D_r1_49*xt46) * (cs49 * rs45);
        J[278] = (-d_D_r1_55*xt46) * (cs55 * rs45);
    }
    {  // row 46
    const T rs46 = nt_rscale<T>(nt_exp_hi(x[46]), fh);
        const T dj46_c0 = D_r1 + T(1);
        const T dj46_c1 = nt_div<T>(xt7, (dj46_c0*dj46_c0));
        J[355] = (nt_div<T>(T(-1), dj46_c0)) * (cs7 * rs46);
        J[358] = (d_D_r1_43*dj46_c1) * (cs43 * rs46);
        J[357] = (d_D_r1_44*dj46_c1) * (cs44 * rs46);
        J[359] = (d_D_r1_47*dj46_c1) * (cs47 * rs46);
        J[360] = (d_D_r1_49*dj46_c1) * (cs49 * rs46);
        J[356] = (d_D_r1_55*dj46_c1) * (cs55 * rs46);
    }
    const T D_r4_c0 = F.h2*K[K_a19] + K[K_a36]*xt8 + K[K_a5]*xt45;
    const T D_r4_c1 = F.o2*K[K_a1] + K[K_a2]*xt46 + T(8.049999999999999e-11)*xt47;
    const T D_r4_c2 = nt_div<T>(T(1), D_r4_c1);
    const T D_r4_c3 = nt_div<T>(D_r4_c0, (D_r4_c1*D_r4_c1));
    const T D_r4 = D_r4_c0*D_r4_c2;
    const T d_D_r4_8 = D_r4_c2*K[K_a36];
    const T d_D_r4_45 = D_r4_c2*K[K_a5];
    const T d_D_r4_46 = -D_r4_c3*K[K_a2];
    const T d_D_r4_47 = -T(8.049999999999999e-11)*D_r4_c3;
    {  // row 55
    const T rs55 = nt_rscale<T>(nt_exp_hi(x[55]), fh);
        J[205] = (-d_D_r4_8*xt43) * (cs8 * rs55);
        J[207] = (-D_r4) * (cs43 * rs55);
        J[206] = (-d_D_r4_45*xt43) * (cs45 * rs55);
        J[209] = (-d_D_r4_46*xt43) * (cs46 * rs55);
        J[208] = (-d_D_r4_47*xt43) * (cs47 * rs55);
    }
    const T D_r7_c0 = F.o2*K[K_b7] + K[K_b6]*xt49;
    const T D_r7 = nt_div<T>(tj[J_no], D_r7_c0);
    const T d_D_r7_49 = nt_div<T>(-K[K_b6]*tj[J_no], (D_r7_c0*D_r7_c0));
    {  // row 51
    const T rs51 = nt_rscale<T>(nt_exp_hi(x[51]), fh);
        J[78] = (-D_r7 - d_D_r7_49*xt49) * (cs49 * rs51);
    }
    const T D_r8_c0 = K[K_b12]*xt48 + tj[J_no3_no2] + tj[J_no3_no];
    const T D_r8_c1 = nt_div<T>(K[K_b9], D_r8_c0);
    const T D_r8 = D_r8_c1*xt46;
    const T d_D_r8_46 = D_r8_c1;
    const T d_D_r8_48 = nt_div<T>(-K[K_b12]*K[K_b9]*xt46, (D_r8_c0*D_r8_c0));
    {  // row 54
    const T rs54 = nt_rscale<T>(nt_exp_hi(x[54]), fh);
        J[68] = T(0);
        J[70] = (-d_D_r8_46*xt48) * (cs46 * rs54);
        J[69] = (-D_r8 - d_D_r8_48*xt48) * (cs48 * rs54);
    }
    const T D_r5_c0 = D_r8*tj[J_no3_no] + K[K_b3]*xt45 + tj[J_no2];
    const T D_r5_c1 = K[K_a26]*xt47 + K[K_b4]*xt46 + K[K_c5]*xt28 + K[K_d4]*xt52 + K[K_e4]*xt53;
    const T D_r5_c2 = nt_div<T>(T(1), D_r5_c1);
    const T D_r5_c3 = nt_div<T>(D_r5_c0, (D_r5_c1*D_r5_c1));
    const T D_r5 = D_r5_c0*D_r5_c2;
    const T d_D_r5_28 = -D_r5_c3*K[K_c5];
    const T d_D_r5_45 = D_r5_c2*K[K_b3];
    const T d_D_r5_46 = D_r5_c2*d_D_r8_46*tj[J_no3_no] - D_r5_c3*K[K_b4];
    const T d_D_r5_47 = -D_r5_c3*K[K_a26];
    const T d_D_r5_48 = D_r5_c2*d_D_r8_48*tj[J_no3_no];
    const T d_D_r5_52 = -D_r5_c3*K[K_d4];
    const T d_D_r5_53 = -D_r5_c3*K[K_e4];
    {  // row 48
    const T rs48 = nt_rscale<T>(nt_exp_hi(x[48]), fh);
        const T dj48_c0 = D_r5*D_r7 + D_r5 + D_r8 + T(1);
        const T dj48_c1 = nt_div<T>(T(1), dj48_c0*dj48_c0);
        const T dj48_c2 = dj48_c1*xt20;
        const T dj48_c3 = dj48_c2*(-D_r7 + T(-1));
        J[270] = (nt_div<T>(T(-1), dj48_c0)) * (cs20 * rs48);
        J[269] = (-d_D_r5_28*dj48_c3) * (cs28 * rs48);
        J[272] = (-d_D_r5_45*dj48_c3) * (cs45 * rs48);
        J[275] = (-d_D_r5_46*dj48_c3 + d_D_r8_46*dj48_c1*xt20) * (cs46 * rs48);
        J[274] = (-d_D_r5_47*dj48_c3) * (cs47 * rs48);
        J[271] = (-d_D_r5_48*dj48_c3 + d_D_r8_48*dj48_c2 + T(1)) * (cs48 * rs48);
        J[276] = (D_r5*d_D_r7_49*dj48_c2) * (cs49 * rs48);
        J[277] = (-d_D_r5_52*dj48_c3) * (cs52 * rs48);
        J[273] = (-d_D_r5_53*dj48_c3) * (cs53 * rs48);
    }
    {  // row 49
    const T rs49 = nt_rscale<T>(nt_exp_hi(x[49]), fh);
        J[361] = (-d_D_r5_28*xt48) * (cs28 * rs49);
        J[363] = (-d_D_r5_45*xt48) * (cs45 * rs49);
        J[366] = (-d_D_r5_46*xt48) * (cs46 * rs49);
        J[365] = (-d_D_r5_47*xt48) * (cs47 * rs49);
        J[362] = (-D_r5 - d_D_r5_48*xt48) * (cs48 * rs49);
        J[367] = (-d_D_r5_52*xt48) * (cs52 * rs49);
        J[364] = (-d_D_r5_53*xt48) * (cs53 * rs49);
    }
    const T D_r6_c0 = F.o2*K[K_a1];
    const T D_r6_c1 = D_r4*D_r6_c0 + K[K_a30]*xt16 + K[K_a6]*xt46 + K[K_c8]*xt27 + K[K_d8]*xt52 + K[K_e10]*xt53;
    const T D_r6_c2 = T(2)*K[K_a27];
    const T D_r6_c3 = D_r6_c2*xt47 + K[K_a17]*xt43 + K[K_a26]*xt49 + K[K_a6b]*xt46 + K[K_a7]*xt45 + K[K_d10]*xt44 + K[K_d33]*xt52 + K[K_d7]*xt44 + K[K_e15]*xt53 + K[K_e7]*xt50 + T(8.049999999999999e-11)*xt55;
    const T D_r6_c4 = nt_div<T>(T(1), D_r6_c3);
    const T D_r6_c5 = D_r6_c0*D_r6_c4;
    const T D_r6_c6 = nt_div<T>(D_r6_c1, (D_r6_c3*D_r6_c3));
    const T D_r6 = D_r6_c1*D_r6_c4;
    const T d_D_r6_8 = D_r6_c5*d_D_r4_8;
    const T d_D_r6_16 = D_r6_c4*K[K_a30];
    const T d_D_r6_27 = D_r6_c4*K[K_c8];
    const T d_D_r6_43 = -D_r6_c6*K[K_a17];
    const T d_D_r6_44 = D_r6_c6*(-K[K_d10] - K[K_d7]);
    const T d_D_r6_45 = D_r6_c5*d_D_r4_45 - D_r6_c6*K[K_a7];
    const T d_D_r6_46 = D_r6_c4*K[K_a6] + D_r6_c5*d_D_r4_46 - D_r6_c6*K[K_a6b];
    const T d_D_r6_47 = -D_r6_c2*D_r6_c6 + D_r6_c5*d_D_r4_47;
    const T d_D_r6_49 = -D_r6_c6*K[K_a26];
    const T d_D_r6_50 = -D_r6_c6*K[K_e7];
    const T d_D_r6_52 = D_r6_c4*K[K_d8] - D_r6_c6*K[K_d33];
    const T d_D_r6_53 = D_r6_c4*K[K_e10] - D_r6_c6*K[K_e15];
    const T d_D_r6_55 = -T(8.049999999999999e-11)*D_r6_c6;
    {  // row 47
    const T rs47 = nt_rscale<T>(nt_exp_hi(x[47]), fh);
        J[342] = (-d_D_r6_8*xt43) * (cs8 * rs47);
        J[343] = (-d_D_r6_16*xt43) * (cs16 * rs47);
        J[345] = (-d_D_r6_27*xt43) * (cs27 * rs47);
        J[350] = (-D_r6 - d_D_r6_43*xt43) * (cs43 * rs47);
        J[347] = (-d_D_r6_44*xt43) * (cs44 * rs47);
        J[346] = (-d_D_r6_45*xt43) * (cs45 * rs47);
        J[352] = (-d_D_r6_46*xt43) * (cs46 * rs47);
        J[351] = (-d_D_r6_47*xt43 + T(1)) * (cs47 * rs47);
        J[353] = (-d_D_r6_49*xt43) * (cs49 * rs47);
        J[349] = (-d_D_r6_50*xt43) * (cs50 * rs47);
        J[354] = (-d_D_r6_52*xt43) * (cs52 * rs47);
        J[348] = (-d_D_r6_53*xt43) * (cs53 * rs47);
        J[344] = (-d_D_r6_55*xt43) * (cs55 * rs47);
    }
    const T D_r13_c0 = K[K_d32]*xt45 + het[0]*xt2 + het[1]*xt12 + tj[J_clono2_cl] + tj[J_clono2_clo];
    const T D_r13_c1 = nt_div<T>(K[K_d31], D_r13_c0);
    const T D_r13_c2 = nt_div<T>(K[K_d31]*xt48, (D_r13_c0*D_r13_c0));
    const T D_r13 = D_r13_c1*xt48;
    const T d_D_r13_2 = -D_r13_c2*het[0];
    const T d_D_r13_12 = -D_r13_c2*het[1];
    const T d_D_r13_45 = -D_r13_c2*K[K_d32];
    const T d_D_r13_48 = D_r13_c1;
    const T D_r9_c0 = D_r13*het[0];
    const T D_r9_c1 = D_r9_c0*xt2 + K[K_d33]*xt47;
    const T D_r9_c2 = K[K_d35]*xt45 + het[4]*xt12 + tj[J_hocl];
    const T D_r9_c3 = nt_div<T>(T(1), D_r9_c2);
    const T D_r9_c4 = D_r9_c3*het[0]*xt2;
    const T D_r9_c5 = nt_div<T>(D_r9_c1, (D_r9_c2*D_r9_c2));
    const T D_r9 = D_r9_c1*D_r9_c3;
    const T d_D_r9_2 = D_r9_c0*D_r9_c3 + D_r9_c4*d_D_r13_2;
    const T d_D_r9_12 = D_r9_c4*d_D_r13_12 - D_r9_c5*het[4];
    const T d_D_r9_45 = D_r9_c3*d_D_r13_45*het[0]*xt2 - D_r9_c5*K[K_d35];
    const T d_D_r9_47 = D_r9_c3*K[K_d33];
    const T d_D_r9_48 = D_r9_c4*d_D_r13_48;
    const T D_r10_c0 = nt_div<T>(K[K_d60], F.hnm*K[K_d61] + tj[J_cl2o2]);
    const T D_r10 = D_r10_c0*xt52;
    const T d_D_r10_52 = D_r10_c0;
    const T D_r12_c0 = nt_div<T>(K[K_e5c], tj[J_brcl]);
    const T D_r12 = D_r12_c0*xt53;
    const T d_D_r12_53 = D_r12_c0;
    const T D_r11_c0 = K[K_d10]*xt47 + K[K_d2]*xt46 + K[K_d37]*xt14 + K[K_d5]*xt1 + K[K_d7]*xt47;
    const T D_r11_c1 = nt_div<T>(T(1), D_r11_c0);
    const T D_r11_c2 = T(2)*tj[J_cl2o2];
    const T D_r11_c3 = D_r10*D_r11_c2 + D_r12*tj[J_brcl] + D_r13*tj[J_clono2_cl] + D_r9*tj[J_hocl] + K[K_c18]*xt28 + K[K_d3]*xt45 + K[K_d4]*xt49 + K[K_d8]*xt43 + K[K_e5b]*xt53;
    const T D_r11_c4 = nt_div<T>(D_r11_c3, (D_r11_c0*D_r11_c0));
    const T D_r11_c5 = D_r11_c1*tj[J_clono2_cl];
    const T D_r11_c6 = D_r11_c1*tj[J_hocl];
    const T D_r11 = D_r11_c1*D_r11_c3;
    const T d_D_r11_1 = -D_r11_c4*K[K_d5];
    const T d_D_r11_2 = D_r11_c5*d_D_r13_2 + D_r11_c6*d_D_r9_2;
    const T d_D_r11_12 = D_r11_c5*d_D_r13_12 + D_r11_c6*d_D_r9_12;
    const T d_D_r11_14 = -D_r11_c4*K[K_d37];
    const T d_D_r11_28 = D_r11_c1*K[K_c18];
    const T d_D_r11_43 = D_r11_c1*K[K_d8];
    const T d_D_r11_45 = D_r11_c1*K[K_d3] + D_r11_c5*d_D_r13_45 + D_r11_c6*d_D_r9_45;
    const T d_D_r11_46 = -D_r11_c4*K[K_d2];
    const T d_D_r11_47 = D_r11_c4*(-K[K_d10] - K[K_d7]) + D_r11_c6*d_D_r9_47;
    const T d_D_r11_48 = D_r11_c5*d_D_r13_48 + D_r11_c6*d_D_r9_48;
    const T d_D_r11_49 = D_r11_c1*K[K_d4];
    const T d_D_r11_52 = D_r11_c1*D_r11_c2*d_D_r10_52;
    const T d_D_r11_53 = D_r11_c1*K[K_e5b] + D_r11_c1*d_D_r12_53*tj[J_brcl];
    {  // row 44
    const T rs44 = nt_rscale<T>(nt_exp_hi(x[44]), fh);
        J[284] = (-d_D_r11_1*xt52) * (cs1 * rs44);
        J[288] = (-d_D_r11_2*xt52) * (cs2 * rs44);
        J[287] = (-d_D_r11_12*xt52) * (cs12 * rs44);
        J[285] = (-d_D_r11_14*xt52) * (cs14 * rs44);
        J[286] = (-d_D_r11_28*xt52) * (cs28 * rs44);
        J[292] = (-d_D_r11_43*xt52) * (cs43 * rs44);
        J[290] = (-d_D_r11_45*xt52) * (cs45 * rs44);
        J[294] = (-d_D_r11_46*xt52) * (cs46 * rs44);
        J[293] = (-d_D_r11_47*xt52) * (cs47 * rs44);
        J[289] = (-d_D_r11_48*xt52) * (cs48 * rs44);
        J[295] = (-d_D_r11_49*xt52) * (cs49 * rs44);
        J[296] = (-D_r11 - d_D_r11_52*xt52) * (cs52 * rs44);
        J[291] = (-d_D_r11_53*xt52) * (cs53 * rs44);
    }
    {  // row 52
    const T rs52 = nt_rscale<T>(nt_exp_hi(x[52]), fh);
        const T dj52_c0 = D_r11 + T(1);
        const T dj52_c1 = nt_div<T>(xt22, (dj52_c0*dj52_c0));
        J[369] = (d_D_r11_1*dj52_c1) * (cs1 * rs52);
        J[373] = (d_D_r11_2*dj52_c1) * (cs2 * rs52);
        J[372] = (d_D_r11_12*dj52_c1) * (cs12 * rs52);
        J[370] = (d_D_r11_14*dj52_c1) * (cs14 * rs52);
        J[368] = (nt_div<T>(T(-1), dj52_c0)) * (cs22 * rs52);
        J[371] = (d_D_r11_28*dj52_c1) * (cs28 * rs52);
        J[377] = (d_D_r11_43*dj52_c1) * (cs43 * rs52);
        J[375] = (d_D_r11_45*dj52_c1) * (cs45 * rs52);
        J[379] = (d_D_r11_46*dj52_c1) * (cs46 * rs52);
        J[378] = (d_D_r11_47*dj52_c1) * (cs47 * rs52);
        J[374] = (d_D_r11_48*dj52_c1) * (cs48 * rs52);
        J[380] = (d_D_r11_49*dj52_c1) * (cs49 * rs52);
        J[381] = (d_D_r11_52*dj52_c1 + T(1)) * (cs52 * rs52);
        J[376] = (d_D_r11_53*dj52_c1) * (cs53 * rs52);
    }
    const T D_r27_c0 = K[K_e8]*xt45 + tj[J_brono2];
    const T D_r27_c1 = nt_div<T>(K[K_e13], D_r27_c0);
    const T D_r27 = D_r27_c1*xt48;
    const T d_D_r27_45 = nt_div<T>(-K[K_e13]*K[K_e8]*xt48, (D_r27_c0*D_r27_c0));
    const T d_D_r27_48 = D_r27_c1;
    const T D_r28_c0 = K[K_e16]*xt45 + tj[J_hobr];
    const T D_r28_c1 = nt_div<T>(K[K_e15], D_r28_c0);
    const T D_r28 = D_r28_c1*xt47;
    const T d_D_r28_45 = nt_div<T>(-K[K_e15]*K[K_e16]*xt47, (D_r28_c0*D_r28_c0));
    const T d_D_r28_47 = D_r28_c1;
    const T D_r29_c0 = nt_div<T>(K[K_e5c], tj[J_brcl]);
    const T D_r29 = D_r29_c0*xt52;
    const T d_D_r29_52 = D_r29_c0;
    const T D_r30_c0 = K[K_c19]*xt27 + K[K_e2]*xt46 + K[K_e7]*xt47;
    const T D_r30_c1 = nt_div<T>(T(1), D_r30_c0);
    const T D_r30_c2 = T(0.85)*tj[J_brono2];
    const T D_r30_c3 = T(2)*K[K_e6];
    const T D_r30_c4 = D_r27*D_r30_c2 + D_r28*tj[J_hobr] + D_r29*tj[J_brcl] + D_r30_c3*xt53 + K[K_e10]*xt43 + K[K_e3]*xt45 + K[K_e4]*xt49 + K[K_e5a]*xt52 + K[K_e5b]*xt52 + tj[J_bro];
    const T D_r30_c5 = nt_div<T>(D_r30_c4, (D_r30_c0*D_r30_c0));
    const T D_r30_c6 = D_r30_c1*D_r30_c2;
    const T D_r30 = D_r30_c1*D_r30_c4;
    const T d_D_r30_27 = -D_r30_c5*K[K_c19];
    const T d_D_r30_43 = D_r30_c1*K[K_e10];
    const T d_D_r30_45 = D_r30_c1*K[K_e3] + D_r30_c1*d_D_r28_45*tj[J_hobr] + D_r30_c6*d_D_r27_45;
    const T d_D_r30_46 = -D_r30_c5*K[K_e2];
    const T d_D_r30_47 = D_r30_c1*d_D_r28_47*tj[J_hobr] - D_r30_c5*K[K_e7];
    const T d_D_r30_48 = D_r30_c6*d_D_r27_48;
    const T d_D_r30_49 = D_r30_c1*K[K_e4];
    const T d_D_r30_52 = D_r30_c1*d_D_r29_52*tj[J_brcl] + D_r30_c1*(K[K_e5a] + K[K_e5b]);
    const T d_D_r30_53 = D_r30_c1*D_r30_c3;
    {  // row 50
    const T rs50 = nt_rscale<T>(nt_exp_hi(x[50]), fh);
        J[307] = (-d_D_r30_27*xt53) * (cs27 * rs50);
        J[311] = (-d_D_r30_43*xt53) * (cs43 * rs50);
        J[309] = (-d_D_r30_45*xt53) * (cs45 * rs50);
        J[313] = (-d_D_r30_46*xt53) * (cs46 * rs50);
        J[312] = (-d_D_r30_47*xt53) * (cs47 * rs50);
        J[308] = (-d_D_r30_48*xt53) * (cs48 * rs50);
        J[314] = (-d_D_r30_49*xt53) * (cs49 * rs50);
        J[315] = (-d_D_r30_52*xt53) * (cs52 * rs50);
        J[310] = (-D_r30 - d_D_r30_53*xt53) * (cs53 * rs50);
    }
    {  // row 53
    const T rs53 = nt_rscale<T>(nt_exp_hi(x[53]), fh);
        const T dj53_c0 = D_r30 + T(1);
        const T dj53_c1 = nt_div<T>(xt23, (dj53_c0*dj53_c0));
        J[297] = (nt_div<T>(T(-1), dj53_c0)) * (cs23 * rs53);
        J[298] = (d_D_r30_27*dj53_c1) * (cs27 * rs53);
        J[302] = (d_D_r30_43*dj53_c1) * (cs43 * rs53);
        J[300] = (d_D_r30_45*dj53_c1) * (cs45 * rs53);
        J[304] = (d_D_r30_46*dj53_c1) * (cs46 * rs53);
        J[303] = (d_D_r30_47*dj53_c1) * (cs47 * rs53);
        J[299] = (d_D_r30_48*dj53_c1) * (cs48 * rs53);
        J[305] = (d_D_r30_49*dj53_c1) * (cs49 * rs53);
        J[306] = (d_D_r30_52*dj53_c1) * (cs52 * rs53);
        J[301] = (d_D_r30_53*dj53_c1 + T(1)) * (cs53 * rs53);
    }
    const T D_coea_c0 = D_r6*K[K_a27];
    const T D_coea_c1 = T(1.7e-11)*D_r4 + T(2)*K[K_a17];
    const T D_coea_c2 = T(1.7e-11)*D_r6;
    const T D_coea_c3 = T(4)*D_coea_c0 + D_coea_c1;
    const T D_coea = D_r6*(T(2)*D_coea_c0 + D_coea_c1) + T(2)*K[K_a31];
    const T d_D_coea_8 = D_coea_c2*d_D_r4_8 + D_coea_c3*d_D_r6_8;
    const T d_D_coea_16 = D_coea_c3*d_D_r6_16;
    const T d_D_coea_27 = D_coea_c3*d_D_r6_27;
    const T d_D_coea_43 = D_coea_c3*d_D_r6_43;
    const T d_D_coea_44 = D_coea_c3*d_D_r6_44;
    const T d_D_coea_45 = D_coea_c2*d_D_r4_45 + D_coea_c3*d_D_r6_45;
    const T d_D_coea_46 = D_coea_c2*d_D_r4_46 + D_coea_c3*d_D_r6_46;
    const T d_D_coea_47 = D_coea_c2*d_D_r4_47 + D_coea_c3*d_D_r6_47;
    const T d_D_coea_49 = D_coea_c3*d_D_r6_49;
    const T d_D_coea_50 = D_coea_c3*d_D_r6_50;
    const T d_D_coea_52 = D_coea_c3*d_D_r6_52;
    const T d_D_coea_53 = D_coea_c3*d_D_r6_53;
    const T d_D_coea_55 = D_coea_c3*d_D_r6_55;
    const T D_coeb_c0 = K[K_b23]*xt48;
    const T D_coeb_c1 = K[K_c7]*xt28;
    const T D_coeb_c2 = K[K_d33]*xt52;
    const T D_coeb_c3 = K[K_d7]*xt44;
    const T D_coeb_c4 = K[K_e15]*xt53;
    const T D_coeb_c5 = K[K_e7]*xt50;
    const T D_coeb_c6 = F.parthbr*K[K_e11];
    const T D_coeb_c7 = F.parthcl*K[K_d11];
    const T D_coeb_c8 = F.parthno3*K[K_b27];
    const T D_coeb_c9 = D_coeb_c0 + D_coeb_c1 + D_coeb_c2 + D_coeb_c3 + D_coeb_c4 + D_coeb_c5;
    const T D_coeb = D_coeb_c0*D_r6 + D_coeb_c1*D_r6 + D_coeb_c2*D_r6 + D_coeb_c3*D_r6 + D_coeb_c4*D_r6 + D_coeb_c5*D_r6 + D_coeb_c6*xt18 + D_coeb_c7*xt12 + D_coeb_c8*xt4 + K[K_b22]*xt48 + K[K_b28]*xt21 + K[K_c17a]*xt29 + K[K_c2]*xt1 + K[K_c8]*xt27 + K[K_d34]*xt14 + K[K_d9]*xt52;
    const T d_D_coeb_1 = K[K_c2];
    const T d_D_coeb_4 = D_coeb_c8;
    const T d_D_coeb_8 = D_coeb_c9*d_D_r6_8;
    const T d_D_coeb_12 = D_coeb_c7;
    const T d_D_coeb_14 = K[K_d34];
    const T d_D_coeb_16 = D_coeb_c9*d_D_r6_16;
    const T d_D_coeb_18 = D_coeb_c6;
    const T d_D_coeb_21 = K[K_b28];
    const T d_D_coeb_27 = D_coeb_c9*d_D_r6_27 + K[K_c8];
    const T d_D_coeb_28 = D_r6*K[K_c7];
    const T d_D_coeb_29 = K[K_c17a];
    const T d_D_coeb_43 = D_coeb_c9*d_D_r6_43;
    const T d_D_coeb_44 = D_coeb_c9*d_D_r6_44 + D_r6*K[K_d7];
    const T d_D_coeb_45 = D_coeb_c9*d_D_r6_45;
    const T d_D_coeb_46 = D_coeb_c9*d_D_r6_46;
    const T d_D_coeb_47 = D_coeb_c9*d_D_r6_47;
    const T d_D_coeb_48 = D_r6*K[K_b23] + K[K_b22];
    const T d_D_coeb_49 = D_coeb_c9*d_D_r6_49;
    const T d_D_coeb_50 = D_coeb_c9*d_D_r6_50 + D_r6*K[K_e7];
    const T d_D_coeb_52 = D_coeb_c9*d_D_r6_52 + D_r6*K[K_d33] + K[K_d9];
    const T d_D_coeb_53 = D_coeb_c9*d_D_r6_53 + D_r6*K[K_e15];
    const T d_D_coeb_55 = D_coeb_c9*d_D_r6_55;
    const T D_coec_c0 = T(2)*tj[J_h2o2];
    const T D_coec_c1 = F.o2*K[K_c15];
    const T D_coec_c2 = F.o2*K[K_c12];
    const T D_coec_c3 = F.h2*K[K_d6];
    const T D_coec_c4 = F.parthno3*tj[J_hno3];
    const T D_coec_c5 = K[K_c3]*xt56;
    const T D_coec_c6 = K[K_e16]*xt45;
    const T D_coec_c7 = F.hnm*K[K_b24] + tj[J_hno4];
    const T D_coec_c8 = K[K_c9]*xt45 + tj[J_ch2o_hco];
    const T D_coec_c9 = K[K_d35]*xt45 + K[K_d37]*xt44 + tj[J_hocl];
    const T D_coec_c10 = K[K_c1a] + K[K_c1b];
    const T D_coec_c11 = D_coec_c10*xt1 + T(2.4e-10)*F.h2;
    const T D_coec_c12 = T(2)*K[K_a1et];
    const T D_coec_c13 = F.parth2o*(D_coec_c12*xt42 + T(2)*tj[J_h2o]);
    const T D_coec = D_ch3o*D_coec_c1 + D_coec_c0*xt16 + D_coec_c11*xt42 + D_coec_c13*xt2 + D_coec_c2*D_hco + D_coec_c3*xt44 + D_coec_c4*xt4 + D_coec_c5*xt45 + D_coec_c6*xt25 + D_coec_c7*xt21 + D_coec_c8*xt27 + D_coec_c9*xt14 + tj[J_ch3o2h]*xt29 + tj[J_hbr]*xt18 + tj[J_hobr]*xt25;
    const T d_D_coec_1 = D_coec_c1*d_D_ch3o_1 + D_coec_c10*xt42;
    const T d_D_coec_2 = D_coec_c13;
    const T d_D_coec_4 = D_coec_c4;
    const T d_D_coec_14 = D_coec_c9;
    const T d_D_coec_16 = D_coec_c0;
    const T d_D_coec_18 = tj[J_hbr];
    const T d_D_coec_21 = D_coec_c7;
    const T d_D_coec_25 = D_coec_c6 + tj[J_hobr];
    const T d_D_coec_27 = D_coec_c2*d_D_hco_27 + D_coec_c8;
    const T d_D_coec_28 = D_coec_c1*d_D_ch3o_28;
    const T d_D_coec_29 = D_coec_c1*d_D_ch3o_29 + tj[J_ch3o2h];
    const T d_D_coec_42 = D_coec_c1*d_D_ch3o_42 + D_coec_c11 + D_coec_c12*F.parth2o*xt2;
    const T d_D_coec_43 = D_coec_c2*d_D_hco_43;
    const T d_D_coec_44 = D_coec_c2*d_D_hco_44 + D_coec_c3 + K[K_d37]*xt14;
    const T d_D_coec_45 = D_coec_c2*d_D_hco_45 + D_coec_c5 + K[K_c9]*xt27 + K[K_d35]*xt14 + K[K_e16]*xt25;
    const T d_D_coec_49 = D_coec_c1*d_D_ch3o_49;
    const T d_D_coec_50 = D_coec_c2*d_D_hco_50;
    const T d_D_coec_52 = D_coec_c1*d_D_ch3o_52;
    const T d_D_coec_56 = K[K_c3]*xt45;
    const T D_argum_c0 = T(4)*D_coea;
    const T D_argum_c1 = D_argum_c0*D_coec + (D_coeb*D_coeb);
    const T D_argum_c2 = T(2)*D_coeb;
    const T D_argum_c3 = T(4)*D_coec;
    const bool sel_D_argum = (D_argum_c1) >= (T(0));
    const T D_argum = sel_D_argum ? T(D_argum_c1) : T(T(0));
    const T d_D_argum_1 = sel_D_argum ? T(D_argum_c0*d_D_coec_1 + D_argum_c2*d_D_coeb_1) : T(T(0));
    const T d_D_argum_2 = sel_D_argum ? T(D_argum_c0*d_D_coec_2) : T(T(0));
    const T d_D_argum_4 = sel_D_argum ? T(D_argum_c0*d_D_coec_4 + D_argum_c2*d_D_coeb_4) : T(T(0));
    const T d_D_argum_8 = sel_D_argum ? T(D_argum_c2*d_D_coeb_8 + D_argum_c3*d_D_coea_8) : T(T(0));
    const T d_D_argum_12 = sel_D_argum ? T(D_argum_c2*d_D_coeb_12) : T(T(0));
    const T d_D_argum_14 = sel_D_argum ? T(D_argum_c0*d_D_coec_14 + D_argum_c2*d_D_coeb_14) : T(T(0));
    const T d_D_argum_16 = sel_D_argum ? T(D_argum_c0*d_D_coec_16 + D_argum_c2*d_D_coeb_16 + D_argum_c3*d_D_coea_16) : T(T(0));
    const T d_D_argum_18 = sel_D_argum ? T(D_argum_c0*d_D_coec_18 + D_argum_c2*d_D_coeb_18) : T(T(0));
    const T d_D_argum_21 = sel_D_argum ? T(D_argum_c0*d_D_coec_21 + D_argum_c2*d_D_coeb_21) : T(T(0));
    const T d_D_argum_25 = sel_D_argum ? T(D_argum_c0*d_D_coec_25) : T(T(0));
    const T d_D_argum_27 = sel_D_argum ? T(D_argum_c0*d_D_coec_27 + D_argum_c2*d_D_coeb_27 + D_argum_c3*d_D_coea_27) : T(T(0));
    const T d_D_argum_28 = sel_D_argum ? T(D_argum_c0*d_D_coec_28 + D_argum_c2*d_D_coeb_28) : T(T(0));
    const T d_D_argum_29 = sel_D_argum ? T(D_argum_c0*d_D_coec_29 + D_argum_c2*d_D_coeb_29) : T(T(0));
    const T d_D_argum_42 = sel_D_argum ? T(D_argum_c0*d_D_coec_42) : T(T(0));
    const T d_D_argum_43 = sel_D_argum ? T(D_argum_c0*d_D_coec_43 + D_argum_c2*d_D_coeb_43 + D_argum_c3*d_D_coea_43) : T(T(0));
    const T d_D_argum_44 = sel_D_argum ? T(D_argum_c0*d_D_coec_44 + D_argum_c2*d_D_coeb_44 + D_argum_c3*d_D_coea_44) : T(T(0));
    const T d_D_argum_45 = sel_D_argum ? T(D_argum_c0*d_D_coec_45 + D_argum_c2*d_D_coeb_45 + D_argum_c3*d_D_coea_45) : T(T(0));
    const T d_D_argum_46 = sel_D_argum ? T(D_argum_c2*d_D_coeb_46 + D_argum_c3*d_D_coea_46) : T(T(0));
    const T d_D_argum_47 = sel_D_argum ? T(D_argum_c2*d_D_coeb_47 + D_argum_c3*d_D_coea_47) : T(T(0));
    const T d_D_argum_48 = sel_D_argum ? T(D_argum_c2*d_D_coeb_48) : T(T(0));
    const T d_D_argum_49 = sel_D_argum ? T(D_argum_c0*d_D_coec_49 + D_argum_c2*d_D_coeb_49 + D_argum_c3*d_D_coea_49) : T(T(0));
    const T d_D_argum_50 = sel_D_argum ? T(D_argum_c0*d_D_coec_50 + D_argum_c2*d_D_coeb_50 + D_argum_c3*d_D_coea_50) : T(T(0));
    const T d_D_argum_52 = sel_D_argum ? T(D_argum_c0*d_D_coec_52 + D_argum_c2*d_D_coeb_52 + D_argum_c3*d_D_coea_52) : T(T(0));
    const T d_D_argum_53 = sel_D_argum ? T(D_argum_c2*d_D_coeb_53 + D_argum_c3*d_D_coea_53) : T(T(0));
    const T d_D_argum_55 = sel_D_argum ? T(D_argum_c2*d_D_coeb_55 + D_argum_c3*d_D_coea_55) : T(T(0));
    const T d_D_argum_56 = sel_D_argum ? T(D_argum_c0*d_D_coec_56) : T(T(0));
    {  // row 43
    const T rs43 = nt_rscale<T>(nt_exp_hi(x[43]), fh);
        const T dj43_c0 = nt_div<T>(T(1), D_coea);
        const T dj43_c1 = nt_div<T>(dj43_c0, T(2));
        const T dj43_c2 = sqrt(D_argum);
        const T dj43_c3 = nt_div<T>(dj43_c0, T(4)*dj43_c2);
        const T dj43_c4 = nt_div<T>(-D_coeb + dj43_c2, T(2)*(D_coea*D_coea));
        J[321] = (-d_D_argum_1*dj43_c3 + d_D_coeb_1*dj43_c1) * (cs1 * rs43);
        J[331] = (-d_D_argum_2*dj43_c3) * (cs2 * rs43);
        J[319] = (-d_D_argum_4*dj43_c3 + d_D_coeb_4*dj43_c1) * (cs4 * rs43);
        J[322] = (-d_D_argum_8*dj43_c3 + d_D_coea_8*dj43_c4 + d_D_coeb_8*dj43_c1) * (cs8 * rs43);
        J[330] = (-d_D_argum_12*dj43_c3 + d_D_coeb_12*dj43_c1) * (cs12 * rs43);
        J[323] = (-d_D_argum_14*dj43_c3 + d_D_coeb_14*dj43_c1) * (cs14 * rs43);
        J[326] = (-d_D_argum_16*dj43_c3 + d_D_coea_16*dj43_c4 + d_D_coeb_16*dj43_c1) * (cs16 * rs43);
        J[325] = (-d_D_argum_18*dj43_c3 + d_D_coeb_18*dj43_c1) * (cs18 * rs43);
        J[320] = (-d_D_argum_21*dj43_c3 + d_D_coeb_21*dj43_c1) * (cs21 * rs43);
        J[317] = (-d_D_argum_25*dj43_c3) * (cs25 * rs43);
        J[329] = (-d_D_argum_27*dj43_c3 + d_D_coea_27*dj43_c4 + d_D_coeb_27*dj43_c1) * (cs27 * rs43);
        J[328] = (-d_D_argum_28*dj43_c3 + d_D_coeb_28*dj43_c1) * (cs28 * rs43);
        J[316] = (-d_D_argum_29*dj43_c3 + d_D_coeb_29*dj43_c1) * (cs29 * rs43);
        J[318] = (-d_D_argum_42*dj43_c3) * (cs42 * rs43);
        J[337] = (-d_D_argum_43*dj43_c3 + d_D_coea_43*dj43_c4 + d_D_coeb_43*dj43_c1 + T(1)) * (cs43 * rs43);
        J[334] = (-d_D_argum_44*dj43_c3 + d_D_coea_44*dj43_c4 + d_D_coeb_44*dj43_c1) * (cs44 * rs43);
        J[333] = (-d_D_argum_45*dj43_c3 + d_D_coea_45*dj43_c4 + d_D_coeb_45*dj43_c1) * (cs45 * rs43);
        J[339] = (-d_D_argum_46*dj43_c3 + d_D_coea_46*dj43_c4 + d_D_coeb_46*dj43_c1) * (cs46 * rs43);
        J[338] = (-d_D_argum_47*dj43_c3 + d_D_coea_47*dj43_c4 + d_D_coeb_47*dj43_c1) * (cs47 * rs43);
        J[332] = (-d_D_argum_48*dj43_c3 + d_D_coeb_48*dj43_c1) * (cs48 * rs43);
        J[340] = (-d_D_argum_49*dj43_c3 + d_D_coea_49*dj43_c4 + d_D_coeb_49*dj43_c1) * (cs49 * rs43);
        J[336] = (-d_D_argum_50*dj43_c3 + d_D_coea_50*dj43_c4 + d_D_coeb_50*dj43_c1) * (cs50 * rs43);
        J[341] = (-d_D_argum_52*dj43_c3 + d_D_coea_52*dj43_c4 + d_D_coeb_52*dj43_c1) * (cs52 * rs43);
        J[335] = (-d_D_argum_53*dj43_c3 + d_D_coea_53*dj43_c4 + d_D_coeb_53*dj43_c1) * (cs53 * rs43);
        J[327] = (-d_D_argum_55*dj43_c3 + d_D_coea_55*dj43_c4 + d_D_coeb_55*dj43_c1) * (cs55 * rs43);
        J[324] = (-d_D_argum_56*dj43_c3) * (cs56 * rs43);
    }
    const T D_t06_c0 = tj[J_hocl]*xt14;
    const T D_t06_c1 = K[K_d33]*xt52;
    const T D_t06_c2 = D_t06_c1*xt47;
    const bool sel_D_t06 = (D_t06_c0) <= (D_t06_c2);
    const T D_t06 = sel_D_t06 ? T(D_t06_c0) : T(D_t06_c2);
    const T d_D_t06_14 = sel_D_t06 ? T(tj[J_hocl]) : T(T(0));
    const T d_D_t06_47 = sel_D_t06 ? T(T(0)) : T(D_t06_c1);
    const T d_D_t06_52 = sel_D_t06 ? T(T(0)) : T(K[K_d33]*xt47);
    const T D_t07_c0 = K[K_e5c]*xt53;
    const T D_t07_c1 = D_t07_c0*xt52;
    const T D_t07_c2 = tj[J_brcl]*xt26;
    const bool sel_D_t07 = (D_t07_c1) <= (D_t07_c2);
    const T D_t07 = sel_D_t07 ? T(D_t07_c1) : T(D_t07_c2);
    const T d_D_t07_26 = sel_D_t07 ? T(T(0)) : T(tj[J_brcl]);
    const T d_D_t07_52 = sel_D_t07 ? T(D_t07_c0) : T(T(0));
    const T d_D_t07_53 = sel_D_t07 ? T(K[K_e5c]*xt52) : T(T(0));
    const T D_t09_c0 = K[K_e15]*xt53;
    const T D_t09_c1 = D_t09_c0*xt47;
    const T D_t09_c2 = tj[J_hobr]*xt25;
    const bool sel_D_t09 = (D_t09_c1) <= (D_t09_c2);
    const T D_t09 = sel_D_t09 ? T(D_t09_c1) : T(D_t09_c2);
    const T d_D_t09_25 = sel_D_t09 ? T(T(0)) : T(tj[J_hobr]);
    const T d_D_t09_47 = sel_D_t09 ? T(D_t09_c0) : T(T(0));
    const T d_D_t09_53 = sel_D_t09 ? T(K[K_e15]*xt47) : T(T(0));
    {  // row 7
    const T rs7 = nt_rscale<T>(nt_exp_hi(x[7]), fh);
        const T dj7_c0 = T(2)*F.dt;
        const T dj7_c1 = nt_div<T>(tj[J_no3_no], fmax(T(1e-30), tj[J_no3_no2] + tj[J_no3_no]));
        const T dj7_c2 = F.dt*xt49;
        const T dj7_c3 = T(2)*K[K_b3];
        const T dj7_c4 = T(2)*K[K_d3];
        const T dj7_c5 = T(2)*K[K_hk3];
        const T dj7_c6 = T(2)*K[K_b9]*dj7_c1;
        const T dj7_c7 = T(2)*K[K_e5b];
        J[105] = (dj7_c0*dj7_c1*tj[J_clono2_cl]) * (cs13 * rs7);
        J[106] = (F.dt*d_D_t06_14) * (cs14 * rs7);
        J[104] = (F.dt*d_D_t09_25) * (cs25 * rs7);
        J[103] = (d_D_t07_26*dj7_c0) * (cs26 * rs7);
        J[108] = (-K[K_c5]*dj7_c2) * (cs28 * rs7);
        J[112] = (F.dt*(K[K_a5]*xt45 + K[K_a6]*xt46)) * (cs43 * rs7);
        J[110] = (F.dt*(K[K_a5]*xt43 + K[K_a7]*xt47 + T(4)*K[K_hk1]*xt45 + dj7_c3*xt48 + dj7_c4*xt52 + dj7_c5*xt46)) * (cs45 * rs7);
        J[114] = (F.dt*(K[K_a2]*xt55 + K[K_a6]*xt43 + K[K_a6b]*xt47 + dj7_c5*xt45 + dj7_c6*xt48)) * (cs46 * rs7);
        J[113] = (F.dt*d_D_t06_47 + F.dt*d_D_t09_47 + F.dt*(K[K_a6b]*xt46 + K[K_a7]*xt45) - K[K_a26]*dj7_c2) * (cs47 * rs7);
        J[109] = (F.dt*(dj7_c3*xt45 + dj7_c6*xt46)) * (cs48 * rs7);
        J[115] = (-F.dt*(K[K_a26]*xt47 + K[K_c5]*xt28)) * (cs49 * rs7);
        J[116] = (F.dt*d_D_t06_52 + F.dt*(nt_div<T>(T(4)*K[K_d60]*tj[J_cl2o2]*xt52, F.hnm*K[K_d61] + tj[J_cl2o2]) + dj7_c4*xt45 + dj7_c7*xt53) + d_D_t07_52*dj7_c0) * (cs52 * rs7);
        J[111] = (F.dt*d_D_t09_53 + F.dt*(T(4)*K[K_e6]*xt53 + dj7_c7*xt52) + d_D_t07_53*dj7_c0) * (cs53 * rs7);
        J[107] = (F.dt*K[K_a2]*xt46) * (cs55 * rs7);
    }
}

// residual rows [1, 8, 11, 12, 13, 14, 17, 19, 20, 23, 24, 25, 27, 28, 29, 31, 33, 35, 36, 39, 42, 43, 45, 50, 51, 52, 53, 54, 55] (day equations, FP64)
template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>
__device__ __forceinline__ void nt_residual_day_w2_0(const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {
    R[1] = -ck0[1] + x[1]*(F.dt*(K[K_c1a]*x[42] + K[K_c1b]*x[42] + K[K_c1c]*x[42] + K[K_c2]*x[43] + K[K_d5]*x[44]) + T(1));
    R[11] = -ck0[11] + x[11];
    R[12] = -F.dt*(K[K_d9]*x[43]*x[52] + x[44]*(F.h2*K[K_d6] + K[K_c10]*x[27] + K[K_d5]*x[1] + K[K_d7]*x[47])) - ck0[12] + x[12]*(F.dt*(F.parthcl*(K[K_d11]*x[43] + tj[J_hcl]) + F.rain_hcl + het[1]*x[13] + het[3]*x[5] + het[4]*x[14] + het[6]*x[25]) + T(1));
    R[13] = -F.dt*K[K_d31]*x[48]*x[52] - ck0[13] + x[13]*(F.dt*(K[K_d32]*x[45] + het[0]*x[2] + het[1]*x[12] + tj[J_clono2_cl] + tj[J_clono2_clo]) + T(1));
    R[14] = -F.dt*(K[K_d33]*x[47]*x[52] + het[0]*x[13]*x[2]) - ck0[14] + x[14]*(F.dt*(K[K_d34]*x[43] + K[K_d35]*x[45] + K[K_d37]*x[44] + het[4]*x[12] + het[8]*x[18] + tj[J_hocl]) + T(1));
    R[17] = -F.dt*(K[K_d36]*x[44]*x[48] + het[3]*x[12]*x[5]) - ck0[17] + x[17]*(F.dt*tj[J_clno2] + T(1));
    R[19] = -F.dt*K[K_e13]*x[48]*x[53] - ck0[19] + x[19]*(F.dt*(K[K_e8]*x[45] + het[5]*x[2] + tj[J_brono2]) + T(1));
    const T dr20_c0 = F.parthno3*x[4];
    R[20] = F.dt*(T(2)*K[K_b6]*x[49]*x[51] + x[48]*(T(2)*K[K_b12]*x[54] + K[K_b22]*x[43] + K[K_b23]*x[47] + K[K_d31]*x[52] + K[K_d36]*x[44] + K[K_e13]*x[53])) - F.dt*(K[K_b27]*dr20_c0*x[43] + T(2)*K[K_b39]*x[0]*x[42] + K[K_d32]*x[13]*x[45] + K[K_e8]*x[19]*x[45] + dr20_c0*tj[J_hno3] + tj[J_brono2]*x[19] + tj[J_clno2]*x[17] + x[13]*(tj[J_clono2_cl] + tj[J_clono2_clo]) + x[21]*(F.hnm*K[K_b24] + K[K_b28]*x[43] + tj[J_hno4]) + x[5]*(T(2)*F.hnm*K[K_b32] + T(2)*tj[J_n2o5])) - ck0[20] + x[20];
    R[23] = F.dt*(K[K_c19]*x[27]*x[50] + K[K_e7]*x[47]*x[50] + x[53]*(K[K_e13]*x[48] + K[K_e15]*x[47] + K[K_e5c]*x[52])) - F.dt*(F.parthbr*x[18]*(K[K_e11]*x[43] + K[K_e9]*x[42] + tj[J_hbr]) + K[K_e16]*x[25]*x[45] + K[K_e8]*x[19]*x[45] + T(2)*het[7]*x[18]*x[25] + tj[J_brcl]*x[26] + tj[J_brono2]*x[19] + tj[J_hobr]*x[25]) - ck0[23] + x[23];
    R[24] = -F.dt*K[K_d60]*(x[52]*x[52]) - ck0[24] + x[24]*(F.dt*(F.hnm*K[K_d61] + tj[J_cl2o2]) + T(1));
    R[25] = -F.dt*(K[K_e15]*x[47]*x[53] + het[5]*x[19]*x[2]) - ck0[25] + x[25]*(F.dt*(K[K_e16]*x[45] + het[6]*x[12] + het[7]*x[18] + tj[J_hobr]) + T(1));
    R[28] = -F.dt*(F.o2*K[K_c4]*x[56] + K[K_c17a]*x[29]*x[43]) - ck0[28] + x[28]*(F.dt*(T(2)*K[K_c14]*x[28] + K[K_c18]*x[52] + K[K_c5]*x[49] + K[K_c7]*x[47]) + T(1));
    R[29] = -F.dt*K[K_c7]*x[28]*x[47] - ck0[29] + x[29]*(F.dt*(K[K_c17a]*x[43] + K[K_c17b]*x[43] + tj[J_ch3o2h]) + T(1));
    R[31] = -ck0[31] + x[31]*(F.dt*(K[K_d91]*x[42] + tj[J_cfc12]) + T(1));
    R[33] = -ck0[33] + x[33]*(F.dt*(K[K_d93]*x[42] + tj[J_ccl4]) + T(1));
    R[35] = -ck0[35] + x[35]*(F.dt*(K[K_d95]*x[43] + tj[J_ch3cl]) + T(1));
    R[36] = -ck0[36] + x[36]*(F.dt*(K[K_d96]*x[42] + K[K_d97]*x[43] + tj[J_hcfc22]) + T(1));
    R[39] = -ck0[39] + x[39]*(F.dt*(K[K_e53]*x[42] + tj[J_h1301]) + T(1));
    R[42] = nt_div<T>(-tj[J_o3_o1d]*x[46], F.n2*K[K_hk4] + F.o2*K[K_hk5]) + x[42];
    const T D_ch3o = nt_div<T>(K[K_c1b]*x[1]*x[42] + tj[J_ch3o2h]*x[29] + x[28]*(T(2)*K[K_c14]*x[28] + K[K_c18]*x[52] + K[K_c5]*x[49]), F.o2*K[K_c15]);
    R[27] = -F.dt*(D_ch3o*F.o2*K[K_c15] + K[K_c17b]*x[29]*x[43] + K[K_c1c]*x[1]*x[42] + K[K_c3]*x[45]*x[56]) - ck0[27] + x[27]*(F.dt*(K[K_c10]*x[44] + K[K_c19]*x[50] + K[K_c8]*x[43] + K[K_c9]*x[45] + tj[J_ch2o_co] + tj[J_ch2o_hco]) + T(1));
    const T D_hco = nt_div<T>(x[27]*(K[K_c10]*x[44] + K[K_c19]*x[50] + K[K_c8]*x[43] + K[K_c9]*x[45] + tj[J_ch2o_hco]), F.o2*K[K_c12]);
    R[8] = -F.dt*(D_hco*F.o2*K[K_c12] + F.co2*tj[J_co2] + tj[J_ch2o_co]*x[27]) - ck0[8] + x[8]*(F.dt*K[K_a36]*x[43] + T(1));
    const T D_r1 = nt_div<T>(K[K_a2]*x[55] + K[K_a6]*x[43] + K[K_a6b]*x[47] + K[K_b4]*x[49] + K[K_d2]*x[44] + tj[J_o3_o1d] + tj[J_o3_o3p], F.o2*K[K_hk2]);
    R[45] = -D_r1*x[46] + x[45];
    const T D_r4 = nt_div<T>(F.h2*K[K_a19] + K[K_a36]*x[8] + K[K_a5]*x[45], F.o2*K[K_a1] + K[K_a2]*x[46] + T(8.049999999999999e-11)*x[47]);
    R[55] = -D_r4*x[43] + x[55];
    const T D_r7 = nt_div<T>(tj[J_no], F.o2*K[K_b7] + K[K_b6]*x[49]);
    R[51] = -D_r7*x[49] + x[51];
    const T D_r8 = nt_div<T>(K[K_b9]*x[46], K[K_b12]*x[48] + tj[J_no3_no2] + tj[J_no3_no]);
    R[54] = -D_r8*x[48] + x[54];
    const T D_r6 = nt_div<T>(D_r4*F.o2*K[K_a1] + K[K_a30]*x[16] + K[K_a6]*x[46] + K[K_c8]*x[27] + K[K_d8]*x[52] + K[K_e10]*x[53], K[K_a17]*x[43] + K[K_a26]*x[49] + T(2)*K[K_a27]*x[47] + K[K_a6b]*x[46] + K[K_a7]*x[45] + K[K_d10]*x[44] + K[K_d33]*x[52] + K[K_d7]*x[44] + K[K_e15]*x[53] + K[K_e7]*x[50] + T(8.049999999999999e-11)*x[55]);
    const T D_r13 = nt_div<T>(K[K_d31]*x[48], K[K_d32]*x[45] + het[0]*x[2] + het[1]*x[12] + tj[J_clono2_cl] + tj[J_clono2_clo]);
    const T D_r9 = nt_div<T>(D_r13*het[0]*x[2] + K[K_d33]*x[47], K[K_d35]*x[45] + het[4]*x[12] + tj[J_hocl]);
    const T D_r10 = nt_div<T>(K[K_d60]*x[52], F.hnm*K[K_d61] + tj[J_cl2o2]);
    const T D_r12 = nt_div<T>(K[K_e5c]*x[53], tj[J_brcl]);
    const T D_r11 = nt_div<T>(T(2)*D_r10*tj[J_cl2o2] + D_r12*tj[J_brcl] + D_r13*tj[J_clono2_cl] + D_r9*tj[J_hocl] + K[K_c18]*x[28] + K[K_d3]*x[45] + K[K_d4]*x[49] + K[K_d8]*x[43] + K[K_e5b]*x[53], K[K_d10]*x[47] + K[K_d2]*x[46] + K[K_d37]*x[14] + K[K_d5]*x[1] + K[K_d7]*x[47]);
    R[52] = nt_div<T>(-x[22], D_r11 + T(1)) + x[52];
    const T D_r27 = nt_div<T>(K[K_e13]*x[48], K[K_e8]*x[45] + tj[J_brono2]);
    const T D_r28 = nt_div<T>(K[K_e15]*x[47], K[K_e16]*x[45] + tj[J_hobr]);
    const T D_r29 = nt_div<T>(K[K_e5c]*x[52], tj[J_brcl]);
    const T D_r30 = nt_div<T>(T(0.85)*D_r27*tj[J_brono2] + D_r28*tj[J_hobr] + D_r29*tj[J_brcl] + K[K_e10]*x[43] + K[K_e3]*x[45] + K[K_e4]*x[49] + K[K_e5a]*x[52] + K[K_e5b]*x[52] + T(2)*K[K_e6]*x[53] + tj[J_bro], K[K_c19]*x[27] + K[K_e2]*x[46] + K[K_e7]*x[47]);
    R[50] = -D_r30*x[53] + x[50];
    R[53] = nt_div<T>(-x[23], D_r30 + T(1)) + x[53];
    const T D_coea = D_r6*(T(1.7e-11)*D_r4 + T(2)*D_r6*K[K_a27] + T(2)*K[K_a17]) + T(2)*K[K_a31];
    const T D_coeb = D_r6*K[K_b23]*x[48] + D_r6*K[K_c7]*x[28] + D_r6*K[K_d33]*x[52] + D_r6*K[K_d7]*x[44] + D_r6*K[K_e15]*x[53] + D_r6*K[K_e7]*x[50] + F.parthbr*K[K_e11]*x[18] + F.parthcl*K[K_d11]*x[12] + F.parthno3*K[K_b27]*x[4] + K[K_b22]*x[48] + K[K_b28]*x[21] + K[K_c17a]*x[29] + K[K_c2]*x[1] + K[K_c8]*x[27] + K[K_d34]*x[14] + K[K_d9]*x[52];
    const T D_coec = D_ch3o*F.o2*K[K_c15] + D_hco*F.o2*K[K_c12] + F.h2*K[K_d6]*x[44] + F.parth2o*x[2]*(T(2)*K[K_a1et]*x[42] + T(2)*tj[J_h2o]) + F.parthno3*tj[J_hno3]*x[4] + K[K_c3]*x[45]*x[56] + K[K_e16]*x[25]*x[45] + tj[J_ch3o2h]*x[29] + T(2)*tj[J_h2o2]*x[16] + tj[J_hbr]*x[18] + tj[J_hobr]*x[25] + x[14]*(K[K_d35]*x[45] + K[K_d37]*x[44] + tj[J_hocl]) + x[21]*(F.hnm*K[K_b24] + tj[J_hno4]) + x[27]*(K[K_c9]*x[45] + tj[J_ch2o_hco]) + x[42]*(T(2.4e-10)*F.h2 + x[1]*(K[K_c1a] + K[K_c1b]));
    const T D_argum_c0 = T(4)*D_coea*D_coec + (D_coeb*D_coeb);
    const bool sel_D_argum = (D_argum_c0) >= (T(0));
    const T D_argum = sel_D_argum ? T(D_argum_c0) : T(T(0));
    R[43] = x[43] + nt_div<T>(-(sqrt(D_argum) - D_coeb), T(2)*D_coea);
}

// scaled Jacobian rows [2, 4, 5, 8, 9, 12, 14, 15, 16, 17, 18, 22, 25, 26, 27, 29, 30, 32, 34, 37, 38, 41, 43, 49, 55] (day equations) into their stored A slots
template <typename T, typename FF, typename PK, typename PJ>
__device__ __forceinline__ void nt_jacobian_day_w2_0(const FF& F, PK K, PK tj, PK het, const double* __restrict__ x, double floor_, PJ J) {
    const int fh = nt_exp_hi(floor_);
    const T xt0 = nt_cvt<T>(x[0]);
    const T xt1 = nt_cvt<T>(x[1]);
    const T xt2 = nt_cvt<T>(x[2]);
    const T xt3 = nt_cvt<T>(x[3]);
    const T xt4 = nt_cvt<T>(x[4]);
    const T xt5 = nt_cvt<T>(x[5]);
    const T xt6 = nt_cvt<T>(x[6]);
    const T xt7 = nt_cvt<T>(x[7]);
    const T xt8 = nt_cvt<T>(x[8]);
    const T xt9 = nt_cvt<T>(x[9]);
    const T xt10 = nt_cvt<T>(x[10]);
    const T xt11 = nt_cvt<T>(x[11]);
    const T xt12 = nt_cvt<T>(x[12]);
    const T xt13 = nt_cvt<T>(x[13]);
    const T xt14 = nt_cvt<T>(x[14]);
    const T xt15 = nt_cvt<T>(x[15]);
    const T xt16 = nt_cvt<T>(x[16]);
    const T xt17 = nt_cvt<T>(x[17]);
    const T xt18 = nt_cvt<T>(x[18]);
    const T xt19 = nt_cvt<T>(x[19]);
    const T xt20 = nt_cvt<T>(x[20]);
    const T xt21 = nt_cvt<T>(x[21]);
    const T xt22 = nt_cvt<T>(x[22]);
    const T xt23 = nt_cvt<T>(x[23]);
    const T xt24 = nt_cvt<T>(x[24]);
    const T xt25 = nt_cvt<T>(x[25]);
    const T xt26 = nt_cvt<T>(x[26]);
    const T xt27 = nt_cvt<T>(x[27]);
    const T xt28 = nt_cvt<T>(x[28]);
    const T xt29 = nt_cvt<T>(x[29]);
    const T xt30 = nt_cvt<T>(x[30]);
    const T xt31 = nt_cvt<T>(x[31]);
    const T xt32 = nt_cvt<T>(x[32]);
    const T xt33 = nt_cvt<T>(x[33]);
    const T xt34 = nt_cvt<T>(x[34]);
    const T xt35 = nt_cvt<T>(x[35]);
    const T xt36 = nt_cvt<T>(x[36]);
    const T xt37 = nt_cvt<T>(x[37]);
    const T xt38 = nt_cvt<T>(x[38]);
    const T xt39 = nt_cvt<T>(x[39]);
    const T xt40 = nt_cvt<T>(x[40]);
    const T xt41 = nt_cvt<T>(x[41]);
    const T xt42 = nt_cvt<T>(x[42]);
    const T xt43 = nt_cvt<T>(x[43]);
    const T xt44 = nt_cvt<T>(x[44]);
    const T xt45 = nt_cvt<T>(x[45]);
    const T xt46 = nt_cvt<T>(x[46]);
    const T xt47 = nt_cvt<T>(x[47]);
    const T xt48 = nt_cvt<T>(x[48]);
    const T xt49 = nt_cvt<T>(x[49]);
    const T xt50 = nt_cvt<T>(x[50]);
    const T xt51 = nt_cvt<T>(x[51]);
    const T xt52 = nt_cvt<T>(x[52]);
    const T xt53 = nt_cvt<T>(x[53]);
    const T xt54 = nt_cvt<T>(x[54]);
    const T xt55 = nt_cvt<T>(x[55]);
    const T xt56 = nt_cvt<T>(x[56]);
    const T cs1 = nt_scale<T>(nt_exp_hi(x[1]), fh);
    const T cs2 = nt_scale<T>(nt_exp_hi(x[2]), fh);
    const T cs4 = nt_scale<T>(nt_exp_hi(x[4]), fh);
    const T cs5 = nt_scale<T>(nt_exp_hi(x[5]), fh);
    const T cs8 = nt_scale<T>(nt_exp_hi(x[8]), fh);
    const T cs9 = nt_scale<T>(nt_exp_hi(x[9]), fh);
    const T cs12 = nt_scale<T>(nt_exp_hi(x[12]), fh);
    const T cs13 = nt_scale<T>(nt_exp_hi(x[13]), fh);
    const T cs14 = nt_scale<T>(nt_exp_hi(x[14]), fh);
    const T cs15 = nt_scale<T>(nt_exp_hi(x[15]), fh);
    const T cs16 = nt_scale<T>(nt_exp_hi(x[16]), fh);
    const T cs17 = nt_scale<T>(nt_exp_hi(x[17]), fh);
    const T cs18 = nt_scale<T>(nt_exp_hi(x[18]), fh);
    const T cs19 = nt_scale<T>(nt_exp_hi(x[19]), fh);
    const T cs21 = nt_scale<T>(nt_exp_hi(x[21]), fh);
    const T cs24 = nt_scale<T>(nt_exp_hi(x[24]), fh);
    const T cs25 = nt_scale<T>(nt_exp_hi(x[25]), fh);
    const T cs26 = nt_scale<T>(nt_exp_hi(x[26]), fh);
    const T cs27 = nt_scale<T>(nt_exp_hi(x[27]), fh);
    const T cs28 = nt_scale<T>(nt_exp_hi(x[28]), fh);
    const T cs29 = nt_scale<T>(nt_exp_hi(x[29]), fh);
    const T cs30 = nt_scale<T>(nt_exp_hi(x[30]), fh);
    const T cs31 = nt_scale<T>(nt_exp_hi(x[31]), fh);
    const T cs32 = nt_scale<T>(nt_exp_hi(x[32]), fh);
    const T cs33 = nt_scale<T>(nt_exp_hi(x[33]), fh);
    const T cs34 = nt_scale<T>(nt_exp_hi(x[34]), fh);
    const T cs35 = nt_scale<T>(nt_exp_hi(x[35]), fh);
    const T cs36 = nt_scale<T>(nt_exp_hi(x[36]), fh);
    const T cs37 = nt_scale<T>(nt_exp_hi(x[37]), fh);
    const T cs38 = nt_scale<T>(nt_exp_hi(x[38]), fh);
    const T cs41 = nt_scale<T>(nt_exp_hi(x[41]), fh);
    const T cs42 = nt_scale<T>(nt_exp_hi(x[42]), fh);
    const T cs43 = nt_scale<T>(nt_exp_hi(x[43]), fh);
    const T cs44 = nt_scale<T>(nt_exp_hi(x[44]), fh);
    const T cs45 = nt_scale<T>(nt_exp_hi(x[45]), fh);
    const T cs46 = nt_scale<T>(nt_exp_hi(x[46]), fh);
    const T cs47 = nt_scale<T>(nt_exp_hi(x[47]), fh);
    const T cs48 = nt_scale<T>(nt_exp_hi(x[48]), fh);
    const T cs49 = nt_scale<T>(nt_exp_hi(x[49]), fh);
    const T cs50 = nt_scale<T>(nt_exp_hi(x[50]), fh);
    const T cs52 = nt_scale<T>(nt_exp_hi(x[52]), fh);
    const T cs53 = nt_scale<T>(nt_exp_hi(x[53]), fh);
    const T cs54 = nt_scale<T>(nt_exp_hi(x[54]), fh);
    const T cs55 = nt_scale<T>(nt_exp_hi(x[55]), fh);
    const T cs56 = nt_scale<T>(nt_exp_hi(x[56]), fh);
    {  // row 2
    const T rs2 = nt_rscale<T>(nt_exp_hi(x[2]), fh);
        const T dj2_c0 = F.dt*xt43;
        const T dj2_c1 = F.dt*F.parth2o;
        const T dj2_c2 = F.parthno3*K[K_b27];
        const T dj2_c3 = F.parthcl*K[K_d11];
        J[261] = (-K[K_c2]*dj2_c0) * (cs1 * rs2);
        J[266] = (dj2_c1*(K[K_a1et]*xt42 + tj[J_h2o]) + T(1)) * (cs2 * rs2);
        J[260] = (-dj2_c0*dj2_c2) * (cs4 * rs2);
        J[265] = (-dj2_c0*dj2_c3) * (cs12 * rs2);
        J[262] = (-K[K_a30]*dj2_c0) * (cs16 * rs2);
        J[264] = (-K[K_c8]*dj2_c0) * (cs27 * rs2);
        J[258] = (-F.dt*(K[K_c17a]*xt43 + K[K_c17b]*xt43)) * (cs29 * rs2);
        J[259] = (K[K_a1et]*dj2_c1*xt2) * (cs42 * rs2);
        J[267] = (-F.dt*(F.h2*K[K_a19] + K[K_a17]*xt47 + K[K_a30]*xt16 + T(2)*K[K_a31]*xt43 + K[K_c17a]*xt29 + K[K_c17b]*xt29 + K[K_c2]*xt1 + K[K_c8]*xt27 + dj2_c2*xt4 + dj2_c3*xt12)) * (cs43 * rs2);
        J[268] = (-F.dt*(K[K_a17]*xt43 + T(1.6e-12)*xt55)) * (cs47 * rs2);
        J[263] = (-T(1.6e-12)*F.dt*xt47) * (cs55 * rs2);
    }
    {  // row 4
    const T rs4 = nt_rscale<T>(nt_exp_hi(x[4]), fh);
        const T dj4_c0 = T(2)*het[2];
        const T dj4_c1 = F.dt*K[K_b22];
        J[122] = (-F.dt*(dj4_c0*xt5 + het[0]*xt13 + het[5]*xt19)) * (cs2 * rs4);
        J[120] = (F.dt*(F.parthno3*(K[K_b27]*xt43 + tj[J_hno3]) + F.rain_hno3) + T(1)) * (cs4 * rs4);
        J[118] = (-F.dt*(dj4_c0*xt2 + het[3]*xt12)) * (cs5 * rs4);
        J[121] = (-F.dt*(het[1]*xt13 + het[3]*xt5)) * (cs12 * rs4);
        J[119] = (-F.dt*(het[0]*xt2 + het[1]*xt12)) * (cs13 * rs4);
        J[117] = (-F.dt*het[5]*xt2) * (cs19 * rs4);
        J[124] = (F.dt*F.parthno3*K[K_b27]*xt4 - dj4_c1*xt48) * (cs43 * rs4);
        J[123] = (-dj4_c1*xt43) * (cs48 * rs4);
    }
    {  // row 5
    const T rs5 = nt_rscale<T>(nt_exp_hi(x[5]), fh);
        const T dj5_c0 = F.dt*xt5;
        const T dj5_c1 = F.dt*K[K_b12];
        J[74] = (dj5_c0*het[2]) * (cs2 * rs5);
        J[72] = (F.dt*(F.hnm*K[K_b32] + het[2]*xt2 + het[3]*xt12 + tj[J_n2o5]) + T(1)) * (cs5 * rs5);
        J[73] = (dj5_c0*het[3]) * (cs12 * rs5);
        J[75] = (-dj5_c1*xt54) * (cs48 * rs5);
        J[71] = (-dj5_c1*xt48) * (cs54 * rs5);
    }
    {  // row 9
    const T rs9 = nt_rscale<T>(nt_exp_hi(x[9]), fh);
        const T dj9_c0 = F.dt*K[K_e5a];
        J[100] = (F.dt*tj[J_oclo] + T(1)) * (cs9 * rs9);
        J[102] = (-dj9_c0*xt53) * (cs52 * rs9);
        J[101] = (-dj9_c0*xt52) * (cs53 * rs9);
    }
    {  // row 12
    const T rs12 = nt_rscale<T>(nt_exp_hi(x[12]), fh);
        const T dj12_c0 = F.dt*xt44;
        const T dj12_c1 = F.dt*xt12;
        const T dj12_c2 = F.dt*K[K_d9];
        J[250] = (-K[K_d5]*dj12_c0) * (cs1 * rs12);
        J[247] = (dj12_c1*het[3]) * (cs5 * rs12);
        J[253] = (F.dt*(F.parthcl*(K[K_d11]*xt43 + tj[J_hcl]) + F.rain_hcl + het[1]*xt13 + het[3]*xt5 + het[4]*xt14 + het[6]*xt25) + T(1)) * (cs12 * rs12);
        J[249] = (dj12_c1*het[1]) * (cs13 * rs12);
        J[251] = (dj12_c1*het[4]) * (cs14 * rs12);
        J[248] = (dj12_c1*het[6]) * (cs25 * rs12);
        J[252] = (-K[K_c10]*dj12_c0) * (cs27 * rs12);
        J[255] = (F.parthcl*K[K_d11]*dj12_c1 - dj12_c2*xt52) * (cs43 * rs12);
        J[254] = (-F.dt*(F.h2*K[K_d6] + K[K_c10]*xt27 + K[K_d5]*xt1 + K[K_d7]*xt47)) * (cs44 * rs12);
        J[256] = (-K[K_d7]*dj12_c0) * (cs47 * rs12);
        J[257] = (-dj12_c2*xt43) * (cs52 * rs12);
    }
    {  // row 14
    const T rs14 = nt_rscale<T>(nt_exp_hi(x[14]), fh);
        const T dj14_c0 = F.dt*het[0];
        const T dj14_c1 = F.dt*xt14;
        const T dj14_c2 = F.dt*K[K_d33];
        J[170] = (-dj14_c0*xt13) * (cs2 * rs14);
        J[169] = (dj14_c1*het[4]) * (cs12 * rs14);
        J[166] = (-dj14_c0*xt2) * (cs13 * rs14);
        J[167] = (F.dt*(K[K_d34]*xt43 + K[K_d35]*xt45 + K[K_d37]*xt44 + het[4]*xt12 + het[8]*xt18 + tj[J_hocl]) + T(1)) * (cs14 * rs14);
        J[168] = (dj14_c1*het[8]) * (cs18 * rs14);
        J[173] = (K[K_d34]*dj14_c1) * (cs43 * rs14);
        J[172] = (K[K_d37]*dj14_c1) * (cs44 * rs14);
        J[171] = (K[K_d35]*dj14_c1) * (cs45 * rs14);
        J[174] = (-dj14_c2*xt52) * (cs47 * rs14);
        J[175] = (-dj14_c2*xt47) * (cs52 * rs14);
    }
    {  // row 15
    const T rs15 = nt_rscale<T>(nt_exp_hi(x[15]), fh);
        J[63] = (-F.dt*(het[1]*xt13 + het[4]*xt14)) * (cs12 * rs15);
        J[61] = (-F.dt*het[1]*xt12) * (cs13 * rs15);
        J[62] = (-F.dt*(K[K_d37]*xt44 + het[4]*xt12)) * (cs14 * rs15);
        J[60] = (F.dt*tj[J_cl2] + T(1)) * (cs15 * rs15);
        J[64] = (-F.dt*K[K_d37]*xt14) * (cs44 * rs15);
        J[65] = (-T(2)*F.dt*K[K_d62]*xt52) * (cs52 * rs15);
    }
    {  // row 16
    const T rs16 = nt_rscale<T>(nt_exp_hi(x[16]), fh);
        J[189] = (F.dt*(F.rain_h2o2 + K[K_a30]*xt43 + tj[J_h2o2]) + T(1)) * (cs16 * rs16);
        J[190] = (F.dt*K[K_a30]*xt16) * (cs43 * rs16);
        J[191] = (-T(2)*F.dt*K[K_a27]*xt47) * (cs47 * rs16);
    }
    {  // row 17
    const T rs17 = nt_rscale<T>(nt_exp_hi(x[17]), fh);
        const T dj17_c0 = F.dt*het[3];
        const T dj17_c1 = F.dt*K[K_d36];
        J[26] = (-dj17_c0*xt12) * (cs5 * rs17);
        J[27] = (-dj17_c0*xt5) * (cs12 * rs17);
        J[25] = (F.dt*tj[J_clno2] + T(1)) * (cs17 * rs17);
        J[29] = (-dj17_c1*xt48) * (cs44 * rs17);
        J[28] = (-dj17_c1*xt44) * (cs48 * rs17);
    }
    {  // row 18
    const T rs18 = nt_rscale<T>(nt_exp_hi(x[18]), fh);
        const T dj18_c0 = F.dt*xt18;
        const T dj18_c1 = F.dt*xt50;
        const T dj18_c2 = F.parthbr*dj18_c0;
        J[183] = (dj18_c0*het[8]) * (cs14 * rs18);
        J[184] = (F.dt*(F.parthbr*(K[K_e11]*xt43 + K[K_e9]*xt42 + tj[J_hbr]) + F.rain_hbr + het[7]*xt25 + het[8]*xt14) + T(1)) * (cs18 * rs18);
        J[181] = (dj18_c0*het[7]) * (cs25 * rs18);
        J[185] = (-K[K_c19]*dj18_c1) * (cs27 * rs18);
        J[182] = (K[K_e9]*dj18_c2) * (cs42 * rs18);
        J[187] = (K[K_e11]*dj18_c2) * (cs43 * rs18);
        J[188] = (-K[K_e7]*dj18_c1) * (cs47 * rs18);
        J[186] = (-F.dt*(K[K_c19]*xt27 + K[K_e7]*xt47)) * (cs50 * rs18);
    }
    {  // row 22
    const T rs22 = nt_rscale<T>(nt_exp_hi(x[22]), fh);
        const T dj22_c0 = F.dt*xt44;
        const T dj22_c1 = T(3)*xt42;
        const T dj22_c2 = T(2)*K[K_d91];
        const T dj22_c3 = T(4)*K[K_d93];
        const T dj22_c4 = T(3)*K[K_d94];
        const T dj22_c5 = F.dt*xt52;
        const T dj22_c6 = T(2)*K[K_d60];
        const T dj22_c7 = T(2)*K[K_d62];
        J[141] = (K[K_d5]*dj22_c0) * (cs1 * rs22);
        J[140] = (-F.dt*tj[J_oclo]) * (cs9 * rs22);
        J[144] = (-F.dt*F.parthcl*(K[K_d11]*xt43 + tj[J_hcl])) * (cs12 * rs22);
        J[135] = (-F.dt*(K[K_d32]*xt45 + tj[J_clono2_cl] + tj[J_clono2_clo])) * (cs13 * rs22);
        J[142] = (-F.dt*(K[K_d34]*xt43 + K[K_d35]*xt45 + tj[J_hocl]) + K[K_d37]*dj22_c0) * (cs14 * rs22);
        J[133] = (-T(2)*F.dt*tj[J_cl2]) * (cs15 * rs22);
        J[128] = (-F.dt*tj[J_clno2]) * (cs17 * rs22);
        J[138] = (-F.dt*(T(2)*F.hnm*K[K_d61] + T(2)*tj[J_cl2o2])) * (cs24 * rs22);
        J[132] = (-F.dt*tj[J_brcl]) * (cs26 * rs22);
        J[143] = (K[K_c10]*dj22_c0) * (cs27 * rs22);
        J[137] = (-F.dt*(K[K_d90]*dj22_c1 + T(3)*tj[J_cfc11])) * (cs30 * rs22);
        J[131] = (-F.dt*(dj22_c2*xt42 + T(2)*tj[J_cfc12])) * (cs31 * rs22);
        J[127] = (-F.dt*(K[K_d92]*dj22_c1 + T(3)*tj[J_cfc113])) * (cs32 * rs22);
        J[129] = (-F.dt*(dj22_c3*xt42 + T(4)*tj[J_ccl4])) * (cs33 * rs22);
        J[136] = (-F.dt*(dj22_c4*xt43 + T(3)*tj[J_ch3ccl3])) * (cs34 * rs22);
        J[134] = (-F.dt*(K[K_d95]*xt43 + tj[J_ch3cl])) * (cs35 * rs22);
        J[130] = (-F.dt*(K[K_d96]*xt42 + K[K_d97]*xt43 + tj[J_hcfc22])) * (cs36 * rs22);
        J[139] = (-F.dt*(T(3)*K[K_d90]*xt30 + T(3)*K[K_d92]*xt32 + K[K_d96]*xt36 + dj22_c2*xt31 + dj22_c3*xt33)) * (cs42 * rs22);
        J[149] = (-F.dt*(F.parthcl*K[K_d11]*xt12 + K[K_d34]*xt14 + K[K_d95]*xt35 + K[K_d97]*xt36 + dj22_c4*xt34) + K[K_d9]*dj22_c5) * (cs43 * rs22);
        J[147] = (F.dt*(F.h2*K[K_d6] + K[K_c10]*xt27 + K[K_d36]*xt48 + K[K_d37]*xt14 + K[K_d5]*xt1 + K[K_d7]*xt47)) * (cs44 * rs22);
        J[146] = (-F.dt*(K[K_d32]*xt13 + K[K_d35]*xt14)) * (cs45 * rs22);
        J[150] = (F.dt*(K[K_d33]*xt52 + K[K_d7]*xt44)) * (cs47 * rs22);
        J[145] = (F.dt*(K[K_d31]*xt52 + K[K_d36]*xt44)) * (cs48 * rs22);
        J[151] = (F.dt*(K[K_d31]*xt48 + K[K_d33]*xt47 + K[K_d9]*xt43 + K[K_e5a]*xt53 + K[K_e5c]*xt53 + dj22_c6*xt52 + dj22_c7*xt52 + xt52*(dj22_c6 + dj22_c7))) * (cs52 * rs22);
        J[148] = (dj22_c5*(K[K_e5a] + K[K_e5c])) * (cs53 * rs22);
    }
    {  // row 25
    const T rs25 = nt_rscale<T>(nt_exp_hi(x[25]), fh);
        const T dj25_c0 = F.dt*het[5];
        const T dj25_c1 = F.dt*xt25;
        const T dj25_c2 = F.dt*K[K_e15];
        J[83] = (-dj25_c0*xt19) * (cs2 * rs25);
        J[82] = (dj25_c1*het[6]) * (cs12 * rs25);
        J[81] = (dj25_c1*het[7]) * (cs18 * rs25);
        J[79] = (-dj25_c0*xt2) * (cs19 * rs25);
        J[80] = (F.dt*(K[K_e16]*xt45 + het[6]*xt12 + het[7]*xt18 + tj[J_hobr]) + T(1)) * (cs25 * rs25);
        J[84] = (K[K_e16]*dj25_c1) * (cs45 * rs25);
        J[86] = (-dj25_c2*xt53) * (cs47 * rs25);
        J[85] = (-dj25_c2*xt47) * (cs53 * rs25);
    }
    {  // row 26
    const T rs26 = nt_rscale<T>(nt_exp_hi(x[26]), fh);
        const T dj26_c0 = F.dt*het[6];
        const T dj26_c1 = F.dt*het[8];
        const T dj26_c2 = F.dt*K[K_e5c];
        J[47] = (-dj26_c0*xt25) * (cs12 * rs26);
        J[45] = (-dj26_c1*xt18) * (cs14 * rs26);
        J[46] = (-dj26_c1*xt14) * (cs18 * rs26);
        J[44] = (-dj26_c0*xt12) * (cs25 * rs26);
        J[43] = (F.dt*tj[J_brcl] + T(1)) * (cs26 * rs26);
        J[49] = (-dj26_c2*xt53) * (cs52 * rs26);
        J[48] = (-dj26_c2*xt52) * (cs53 * rs26);
    }
    {  // row 29
    const T rs29 = nt_rscale<T>(nt_exp_hi(x[29]), fh);
        const T dj29_c0 = F.dt*K[K_c7];
        J[35] = (-dj29_c0*xt47) * (cs28 * rs29);
        J[34] = (F.dt*(K[K_c17a]*xt43 + K[K_c17b]*xt43 + tj[J_ch3o2h]) + T(1)) * (cs29 * rs29);
        J[36] = (F.dt*xt29*(K[K_c17a] + K[K_c17b])) * (cs43 * rs29);
        J[37] = (-dj29_c0*xt28) * (cs47 * rs29);
    }
    {  // row 30
    const T rs30 = nt_rscale<T>(nt_exp_hi(x[30]), fh);
        J[95] = (F.dt*(K[K_d90]*xt42 + tj[J_cfc11]) + T(1)) * (cs30 * rs30);
        J[96] = (F.dt*K[K_d90]*xt30) * (cs42 * rs30);
    }
    {  // row 32
    const T rs32 = nt_rscale<T>(nt_exp_hi(x[32]), fh);
        J[18] = (F.dt*(K[K_d92]*xt42 + tj[J_cfc113]) + T(1)) * (cs32 * rs32);
        J[19] = (F.dt*K[K_d92]*xt32) * (cs42 * rs32);
    }
    {  // row 34
    const T rs34 = nt_rscale<T>(nt_exp_hi(x[34]), fh);
        J[93] = (F.dt*(K[K_d94]*xt43 + tj[J_ch3ccl3]) + T(1)) * (cs34 * rs34);
        J[94] = (F.dt*K[K_d94]*xt34) * (cs43 * rs34);
    }
    {  // row 37
    const T rs37 = nt_rscale<T>(nt_exp_hi(x[37]), fh);
        const T dj37_c0 = F.dt*xt37;
        J[52] = (F.dt*(K[K_e50]*xt42 + K[K_e51]*xt43 + tj[J_ch3br]) + T(1)) * (cs37 * rs37);
        J[53] = (K[K_e50]*dj37_c0) * (cs42 * rs37);
        J[54] = (K[K_e51]*dj37_c0) * (cs43 * rs37);
    }
    {  // row 38
    const T rs38 = nt_rscale<T>(nt_exp_hi(x[38]), fh);
        J[30] = (F.dt*(K[K_e52]*xt42 + tj[J_h1211]) + T(1)) * (cs38 * rs38);
        J[31] = (F.dt*K[K_e52]*xt38) * (cs42 * rs38);
    }
    {  // row 41
    const T rs41 = nt_rscale<T>(nt_exp_hi(x[41]), fh);
        J[125] = (F.dt*(K[K_e54]*xt43 + tj[J_ch2br2]) + T(1)) * (cs41 * rs41);
        J[126] = (F.dt*K[K_e54]*xt41) * (cs43 * rs41);
    }
    const T D_ch3o_c0 = K[K_c1b]*xt42;
    const T D_ch3o_c1 = K[K_c14]*xt28;
    const T D_ch3o_c2 = K[K_c18]*xt52 + K[K_c5]*xt49;
    const T D_ch3o_c3 = nt_div<T>(T(1), F.o2*K[K_c15]);
    const T D_ch3o_c4 = D_ch3o_c3*xt28;
    const T D_ch3o = D_ch3o_c3*(D_ch3o_c0*xt1 + tj[J_ch3o2h]*xt29 + xt28*(T(2)*D_ch3o_c1 + D_ch3o_c2));
    const T d_D_ch3o_1 = D_ch3o_c0*D_ch3o_c3;
    const T d_D_ch3o_28 = D_ch3o_c3*(T(4)*D_ch3o_c1 + D_ch3o_c2);
    const T d_D_ch3o_29 = D_ch3o_c3*tj[J_ch3o2h];
    const T d_D_ch3o_42 = D_ch3o_c3*K[K_c1b]*xt1;
    const T d_D_ch3o_49 = D_ch3o_c4*K[K_c5];
    const T d_D_ch3o_52 = D_ch3o_c4*K[K_c18];
    {  // row 27
    const T rs27 = nt_rscale<T>(nt_exp_hi(x[27]), fh);
        const T dj27_c0 = F.dt*K[K_c1c];
        const T dj27_c1 = F.dt*F.o2*K[K_c15];
        const T dj27_c2 = F.dt*K[K_c17b];
        const T dj27_c3 = F.dt*xt27;
        const T dj27_c4 = F.dt*K[K_c3];
        J[219] = (-d_D_ch3o_1*dj27_c1 - dj27_c0*xt42) * (cs1 * rs27);
        J[222] = (F.dt*(K[K_c10]*xt44 + K[K_c19]*xt50 + K[K_c8]*xt43 + K[K_c9]*xt45 + tj[J_ch2o_co] + tj[J_ch2o_hco]) + T(1)) * (cs27 * rs27);
        J[221] = (-d_D_ch3o_28*dj27_c1) * (cs28 * rs27);
        J[217] = (-d_D_ch3o_29*dj27_c1 - dj27_c2*xt43) * (cs29 * rs27);
        J[218] = (-d_D_ch3o_42*dj27_c1 - dj27_c0*xt1) * (cs42 * rs27);
        J[226] = (F.dt*K[K_c8]*xt27 - dj27_c2*xt29) * (cs43 * rs27);
        J[224] = (K[K_c10]*dj27_c3) * (cs44 * rs27);
        J[223] = (F.dt*K[K_c9]*xt27 - dj27_c4*xt56) * (cs45 * rs27);
        J[227] = (-d_D_ch3o_49*dj27_c1) * (cs49 * rs27);
        J[225] = (K[K_c19]*dj27_c3) * (cs50 * rs27);
        J[228] = (-d_D_ch3o_52*dj27_c1) * (cs52 * rs27);
        J[220] = (-dj27_c4*xt45) * (cs56 * rs27);
    }
    const T D_hco_c0 = nt_div<T>(T(1), F.o2*K[K_c12]);
    const T D_hco_c1 = D_hco_c0*(K[K_c10]*xt44 + K[K_c19]*xt50 + K[K_c8]*xt43 + K[K_c9]*xt45 + tj[J_ch2o_hco]);
    const T D_hco_c2 = D_hco_c0*xt27;
    const T D_hco = D_hco_c1*xt27;
    const T d_D_hco_27 = D_hco_c1;
    const T d_D_hco_43 = D_hco_c2*K[K_c8];
    const T d_D_hco_44 = D_hco_c2*K[K_c10];
    const T d_D_hco_45 = D_hco_c2*K[K_c9];
    const T d_D_hco_50 = D_hco_c2*K[K_c19];
    {  // row 8
    const T rs8 = nt_rscale<T>(nt_exp_hi(x[8]), fh);
        const T dj8_c0 = F.dt*F.o2*K[K_c12];
        J[160] = (F.dt*K[K_a36]*xt43 + T(1)) * (cs8 * rs8);
        J[161] = (-F.dt*tj[J_ch2o_co] - d_D_hco_27*dj8_c0) * (cs27 * rs8);
        J[165] = (F.dt*K[K_a36]*xt8 - d_D_hco_43*dj8_c0) * (cs43 * rs8);
        J[163] = (-d_D_hco_44*dj8_c0) * (cs44 * rs8);
        J[162] = (-d_D_hco_45*dj8_c0) * (cs45 * rs8);
        J[164] = (-d_D_hco_50*dj8_c0) * (cs50 * rs8);
    }
    const T D_r4_c0 = F.h2*K[K_a19] + K[K_a36]*xt8 + K[K_a5]*xt45;
    const T D_r4_c1 = F.o2*K[K_a1] + K[K_a2]*xt46 + T(8.049999999999999e-11)*xt47;
    const T D_r4_c2 = nt_div<T>(T(1), D_r4_c1);
    const T D_r4_c3 = nt_div<T>(D_r4_c0, (D_r4_c1*D_r4_c1));
    const T D_r4 = D_r4_c0*D_r4_c2;
    const T d_D_r4_8 = D_r4_c2*K[K_a36];
    const T d_D_r4_45 = D_r4_c2*K[K_a5];
    const T d_D_r4_46 = -D_r4_c3*K[K_a2];
    const T d_D_r4_47 = -T(8.049999999999999e-11)*D_r4_c3;
    {  // row 55
    const T rs55 = nt_rscale<T>(nt_exp_hi(x[55]), fh);
        J[205] = (-d_D_r4_8*xt43) * (cs8 * rs55);
        J[207] = (-D_r4) * (cs43 * rs55);
        J[206] = (-d_D_r4_45*xt43) * (cs45 * rs55);
        J[209] = (-d_D_r4_46*xt43) * (cs46 * rs55);
        J[208] = (-d_D_r4_47*xt43) * (cs47 * rs55);
    }
    const T D_r8_c0 = K[K_b12]*xt48 + tj[J_no3_no2] + tj[J_no3_no];
    const T D_r8_c1 = nt_div<T>(K[K_b9], D_r8_c0);
    const T D_r8 = D_r8_c1*xt46;
    const T d_D_r8_46 = D_r8_c1;
    const T d_D_r8_48 = nt_div<T>(-K[K_b12]*K[K_b9]*xt46, (D_r8_c0*D_r8_c0));
    const T D_r5_c0 = D_r8*tj[J_no3_no] + K[K_b3]*xt45 + tj[J_no2];
    const T D_r5_c1 = K[K_a26]*xt47 + K[K_b4]*xt46 + K[K_c5]*xt28 + K[K_d4]*xt52 + K[K_e4]*xt53;
    const T D_r5_c2 = nt_div<T>(T(1), D_r5_c1);
    const T D_r5_c3 = nt_div<T>(D_r5_c0, (D_r5_c1*D_r5_c1));
    const T D_r5 = D_r5_c0*D_r5_c2;
    const T d_D_r5_28 = -D_r5_c3*K[K_c5];
    const T d_D_r5_45 = D_r5_c2*K[K_b3];
    const T d_D_r5_46 = D_r5_c2*d_D_r8_46*tj[J_no3_no] - D_r5_c3*K[K_b4];
    const T d_D_r5_47 = -D_r5_c3*K[K_a26];
    const T d_D_r5_48 = D_r5_c2*d_D_r8_48*tj[J_no3_no];
    const T d_D_r5_52 = -D_r5_c3*K[K_d4];
    const T d_D_r5_53 = -D_r5_c3*K[K_e4];
    {  // row 49
    const T rs49 = nt_rscale<T>(nt_exp_hi(x[49]), fh);
        J[361] = (-d_D_r5_28*xt48) * (cs28 * rs49);
        J[363] = (-d_D_r5_45*xt48) * (cs45 * rs49);
        J[366] = (-d_D_r5_46*xt48) * (cs46 * rs49);
        J[365] = (-d_D_r5_47*xt48) * (cs47 * rs49);
        J[362] = (-D_r5 - d_D_r5_48*xt48) * (cs48 * rs49);
        J[367] = (-d_D_r5_52*xt48) * (cs52 * rs49);
        J[364] = (-d_D_r5_53*xt48) * (cs53 * rs49);
    }
    const T D_r6_c0 = F.o2*K[K_a1];
    const T D_r6_c1 = D_r4*D_r6_c0 + K[K_a30]*xt16 + K[K_a6]*xt46 + K[K_c8]*xt27 + K[K_d8]*xt52 + K[K_e10]*xt53;
    const T D_r6_c2 = T(2)*K[K_a27];
    const T D_r6_c3 = D_r6_c2*xt47 + K[K_a17]*xt43 + K[K_a26]*xt49 + K[K_a6b]*xt46 + K[K_a7]*xt45 + K[K_d10]*xt44 + K[K_d33]*xt52 + K[K_d7]*xt44 + K[K_e15]*xt53 + K[K_e7]*xt50 + T(8.049999999999999e-11)*xt55;
    const T D_r6_c4 = nt_div<T>(T(1), D_r6_c3);
    const T D_r6_c5 = D_r6_c0*D_r6_c4;
    const T D_r6_c6 = nt_div<T>(D_r6_c1, (D_r6_c3*D_r6_c3));
    const T D_r6 = D_r6_c1*D_r6_c4;
    const T d_D_r6_8 = D_r6_c5*d_D_r4_8;
    const T d_D_r6_16 = D_r6_c4*K[K_a30];
    const T d_D_r6_27 = D_r6_c4*K[K_c8];
    const T d_D_r6_43 = -D_r6_c6*K[K_a17];
    const T d_D_r6_44 = D_r6_c6*(-K[K_d10] - K[K_d7]);
    const T d_D_r6_45 = D_r6_c5*d_D_r4_45 - D_r6_c6*K[K_a7];
    const T d_D_r6_46 = D_r6_c4*K[K_a6] + D_r6_c5*d_D_r4_46 - D_r6_c6*K[K_a6b];
    const T d_D_r6_47 = -D_r6_c2*D_r6_c6 + D_r6_c5*d_D_r4_47;
    const T d_D_r6_49 = -D_r6_c6*K[K_a26];
    const T d_D_r6_50 = -D_r6_c6*K[K_e7];
    const T d_D_r6_52 = D_r6_c4*K[K_d8] - D_r6_c6*K[K_d33];
    const T d_D_r6_53 = D_r6_c4*K[K_e10] - D_r6_c6*K[K_e15];
    const T d_D_r6_55 = -T(8.049999999999999e-11)*D_r6_c6;
    const T D_coea_c0 = D_r6*K[K_a27];
    const T D_coea_c1 = T(1.7e-11)*D_r4 + T(2)*K[K_a17];
    const T D_coea_c2 = T(1.7e-11)*D_r6;
    const T D_coea_c3 = T(4)*D_coea_c0 + D_coea_c1;
    const T D_coea = D_r6*(T(2)*D_coea_c0 + D_coea_c1) + T(2)*K[K_a31];
    const T d_D_coea_8 = D_coea_c2*d_D_r4_8 + D_coea_c3*d_D_r6_8;
    const T d_D_coea_16 = D_coea_c3*d_D_r6_16;
    const T d_D_coea_27 = D_coea_c3*d_D_r6_27;
    const T d_D_coea_43 = D_coea_c3*d_D_r6_43;
    const T d_D_coea_44 = D_coea_c3*d_D_r6_44;
    const T d_D_coea_45 = D_coea_c2*d_D_r4_45 + D_coea_c3*d_D_r6_45;
    const T d_D_coea_46 = D_coea_c2*d_D_r4_46 + D_coea_c3*d_D_r6_46;
    const T d_D_coea_47 = D_coea_c2*d_D_r4_47 + D_coea_c3*d_D_r6_47;
    const T d_D_coea_49 = D_coea_c3*d_D_r6_49;
    const T d_D_coea_50 = D_coea_c3*d_D_r6_50;
    const T d_D_coea_52 = D_coea_c3*d_D_r6_52;
    const T d_D_coea_53 = D_coea_c3*d_D_r6_53;
    const T d_D_coea_55 = D_coea_c3*d_D_r6_55;
    const T D_coeb_c0 = K[K_b23]*xt48;
    const T D_coeb_c1 = K[K_c7]*xt28;
    const T D_coeb_c2 = K[K_d33]*xt52;
    const T D_coeb_c3 = K[K_d7]*xt44;
    const T D_coeb_c4 = K[K_e15]*xt53;
    const T D_coeb_c5 = K[K_e7]*xt50;
    const T D_coeb_c6 = F.parthbr*K[K_e11];
    const T D_coeb_c7 = F.parthcl*K[K_d11];
    const T D_coeb_c8 = F.parthno3*K[K_b27];
    const T D_coeb_c9 = D_coeb_c0 + D_coeb_c1 + D_coeb_c2 + D_coeb_c3 + D_coeb_c4 + D_coeb_c5;
    const T D_coeb = D_coeb_c0*D_r6 + D_coeb_c1*D_r6 + D_coeb_c2*D_r6 + D_coeb_c3*D_r6 + D_coeb_c4*D_r6 + D_coeb_c5*D_r6 + D_coeb_c6*xt18 + D_coeb_c7*xt12 + D_coeb_c8*xt4 + K[K_b22]*xt48 + K[K_b28]*xt21 + K[K_c17a]*xt29 + K[K_c2]*xt1 + K[K_c8]*xt27 + K[K_d34]*xt14 + K[K_d9]*xt52;
    const T d_D_coeb_1 = K[K_c2];
    const T d_D_coeb_4 = D_coeb_c8;
    const T d_D_coeb_8 = D_coeb_c9*d_D_r6_8;
    const T d_D_coeb_12 = D_coeb_c7;
    const T d_D_coeb_14 = K[K_d34];
    const T d_D_coeb_16 = D_coeb_c9*d_D_r6_16;
    const T d_D_coeb_18 = D_coeb_c6;
    const T d_D_coeb_21 = K[K_b28];
    const T d_D_coeb_27 = D_coeb_c9*d_D_r6_27 + K[K_c8];
    const T d_D_coeb_28 = D_r6*K[K_c7];
    const T d_D_coeb_29 = K[K_c17a];
    const T d_D_coeb_43 = D_coeb_c9*d_D_r6_43;
    const T d_D_coeb_44 = D_coeb_c9*d_D_r6_44 + D_r6*K[K_d7];
    const T d_D_coeb_45 = D_coeb_c9*d_D_r6_45;
    const T d_D_coeb_46 = D_coeb_c9*d_D_r6_46;
    const T d_D_coeb_47 = D_coeb_c9*d_D_r6_47;
    const T d_D_coeb_48 = D_r6*K[K_b23] + K[K_b22];
    const T d_D_coeb_49 = D_coeb_c9*d_D_r6_49;
    const T d_D_coeb_50 = D_coeb_c9*d_D_r6_50 + D_r6*K[K_e7];
    const T d_D_coeb_52 = D_coeb_c9*d_D_r6_52 + D_r6*K[K_d33] + K[K_d9];
    const T d_D_coeb_53 = D_coeb_c9*d_D_r6_53 + D_r6*K[K_e15];
    const T d_D_coeb_55 = D_coeb_c9*d_D_r6_55;
    const T D_coec_c0 = T(2)*tj[J_h2o2];
    const T D_coec_c1 = F.o2*K[K_c15];
    const T D_coec_c2 = F.o2*K[K_c12];
    const T D_coec_c3 = F.h2*K[K_d6];
    const T D_coec_c4 = F.parthno3*tj[J_hno3];
    const T D_coec_c5 = K[K_c3]*xt56;
    const T D_coec_c6 = K[K_e16]*xt45;
    const T D_coec_c7 = F.hnm*K[K_b24] + tj[J_hno4];
    const T D_coec_c8 = K[K_c9]*xt45 + tj[J_ch2o_hco];
    const T D_coec_c9 = K[K_d35]*xt45 + K[K_d37]*xt44 + tj[J_hocl];
    const T D_coec_c10 = K[K_c1a] + K[K_c1b];
    const T D_coec_c11 = D_coec_c10*xt1 + T(2.4e-10)*F.h2;
    const T D_coec_c12 = T(2)*K[K_a1et];
    const T D_coec_c13 = F.parth2o*(D_coec_c12*xt42 + T(2)*tj[J_h2o]);
    const T D_coec = D_ch3o*D_coec_c1 + D_coec_c0*xt16 + D_coec_c11*xt42 + D_coec_c13*xt2 + D_coec_c2*D_hco + D_coec_c3*xt44 + D_coec_c4*xt4 + D_coec_c5*xt45 + D_coec_c6*xt25 + D_coec_c7*xt21 + D_coec_c8*xt27 + D_coec_c9*xt14 + tj[J_ch3o2h]*xt29 + tj[J_hbr]*xt18 + tj[J_hobr]*xt25;
    const T d_D_coec_1 = D_coec_c1*d_D_ch3o_1 + D_coec_c10*xt42;
    const T d_D_coec_2 = D_coec_c13;
    const T d_D_coec_4 = D_coec_c4;
    const T d_D_coec_14 = D_coec_c9;
    const T d_D_coec_16 = D_coec_c0;
    const T d_D_coec_18 = tj[J_hbr];
    const T d_D_coec_21 = D_coec_c7;
    const T d_D_coec_25 = D_coec_c6 + tj[J_hobr];
    const T d_D_coec_27 = D_coec_c2*d_D_hco_27 + D_coec_c8;
    const T d_D_coec_28 = D_coec_c1*d_D_ch3o_28;
    const T d_D_coec_29 = D_coec_c1*d_D_ch3o_29 + tj[J_ch3o2h];
    const T d_D_coec_42 = D_coec_c1*d_D_ch3o_42 + D_coec_c11 + D_coec_c12*F.parth2o*xt2;
    const T d_D_coec_43 = D_coec_c2*d_D_hco_43;
    const T d_D_coec_44 = D_coec_c2*d_D_hco_44 + D_coec_c3 + K[K_d37]*xt14;
    const T d_D_coec_45 = D_coec_c2*d_D_hco_45 + D_coec_c5 + K[K_c9]*xt27 + K[K_d35]*xt14 + K[K_e16]*xt25;
    const T d_D_coec_49 = D_coec_c1*d_D_ch3o_49;
    const T d_D_coec_50 = D_coec_c2*d_D_hco_50;
    const T d_D_coec_52 = D_coec_c1*d_D_ch3o_52;
    const T d_D_coec_56 = K[K_c3]*xt45;
    const T D_argum_c0 = T(4)*D_coea;
    const T D_argum_c1 = D_argum_c0*D_coec + (D_coeb*D_coeb);
    const T D_argum_c2 = T(2)*D_coeb;
    const T D_argum_c3 = T(4)*D_coec;
    const bool sel_D_argum = (D_argum_c1) >= (T(0));
    const T D_argum = sel_D_argum ? T(D_argum_c1) : T(T(0));
    const T d_D_argum_1 = sel_D_argum ? T(D_argum_c0*d_D_coec_1 + D_argum_c2*d_D_coeb_1) : T(T(0));
    const T d_D_argum_2 = sel_D_argum ? T(D_argum_c0*d_D_coec_2) : T(T(0));
    const T d_D_argum_4 = sel_D_argum ? T(D_argum_c0*d_D_coec_4 + D_argum_c2*d_D_coeb_4) : T(T(0));
    const T d_D_argum_8 = sel_D_argum ? T(D_argum_c2*d_D_coeb_8 + D_argum_c3*d_D_coea_8) : T(T(0));
    const T d_D_argum_12 = sel_D_argum ? T(D_argum_c2*d_D_coeb_12) : T(T(0));
    const T d_D_argum_14 = sel_D_argum ? T(D_argum_c0*d_D_coec_14 + D_argum_c2*d_D_coeb_14) : T(T(0));
    const T d_D_argum_16 = sel_D_argum ? T(D_argum_c0*d_D_coec_16 + D_argum_c2*d_D_coeb_16 + D_argum_c3*d_D_coea_16) : T(T(0));
    const T d_D_argum_18 = sel_D_argum ? T(D_argum_c0*d_D_coec_18 + D_argum_c2*d_D_coeb_18) : T(T(0));
    const T d_D_argum_21 = sel_D_argum ? T(D_argum_c0*d_D_coec_21 + D_argum_c2*d_D_coeb_21) : T(T(0));
    const T d_D_argum_25 = sel_D_argum ? T(D_argum_c0*d_D_coec_25) : T(T(0));
    const T d_D_argum_27 = sel_D_argum ? T(D_argum_c0*d_D_coec_27 + D_argum_c2*d_D_coeb_27 + D_argum_c3*d_D_coea_27) : T(T(0));
    const T d_D_argum_28 = sel_D_argum ? T(D_argum_c0*d_D_coec_28 + D_argum_c2*d_D_coeb_28) : T(T(0));
    const T d_D_argum_29 = sel_D_argum ? T(D_argum_c0*d_D_coec_29 + D_argum_c2*d_D_coeb_29) : T(T(0));
    const T d_D_argum_42 = sel_D_argum ? T(D_argum_c0*d_D_coec_42) : T(T(0));
    const T d_D_argum_43 = sel_D_argum ? T(D_argum_c0*d_D_coec_43 + D_argum_c2*d_D_coeb_43 + D_argum_c3*d_D_coea_43) : T(T(0));
    const T d_D_argum_44 = sel_D_argum ? T(D_argum_c0*d_D_coec_44 + D_argum_c2*d_D_coeb_44 + D_argum_c3*d_D_coea_44) : T(T(0));
    const T d_D_argum_45 = sel_D_argum ? T(D_argum_c0*d_D_coec_45 + D_argum_c2*d_D_coeb_45 + D_argum_c3*d_D_coea_45) : T(T(0));
    const T d_D_argum_46 = sel_D_argum ? T(D_argum_c2*d_D_coeb_46 + D_argum_c3*d_D_coea_46) : T(T(0));
    const T d_D_argum_47 = sel_D_argum ? T(D_argum_c2*d_D_coeb_47 + D_argum_c3*d_D_coea_47) : T(T(0));
    const T d_D_argum_48 = sel_D_argum ? T(D_argum_c2*d_D_coeb_48) : T(T(0));
    const T d_D_argum_49 = sel_D_argum ? T(D_argum_c0*d_D_coec_49 + D_argum_c2*d_D_coeb_49 + D_argum_c3*d_D_coea_49) : T(T(0));
    const T d_D_argum_50 = sel_D_argum ? T(D_argum_c0*d_D_coec_50 + D_argum_c2*d_D_coeb_50 + D_argum_c3*d_D_coea_50) : T(T(0));
    const T d_D_argum_52 = sel_D_argum ? T(D_argum_c0*d_D_coec_52 + D_argum_c2*d_D_coeb_52 + D_argum_c3*d_D_coea_52) : T(T(0));
    const T d_D_argum_53 = sel_D_argum ? T(D_argum_c2*d_D_coeb_53 + D_argum_c3*d_D_coea_53) : T(T(0));
    const T d_D_argum_55 = sel_D_argum ? T(D_argum_c2*d_D_coeb_55 + D_argum_c3*d_D_coea_55) : T(T(0));
    const T d_D_argum_56 = sel_D_argum ? T(D_argum_c0*d_D_coec_56) : T(T(0));
    {  // row 43
    const T rs43 = nt_rscale<T>(nt_exp_hi(x[43]), fh);
        const T dj43_c0 = nt_div<T>(T(1), D_coea);
        const T dj43_c1 = nt_div<T>(dj43_c0, T(2));
        const T dj43_c2 = sqrt(D_argum);
        const T dj43_c3 = nt_div<T>(dj43_c0, T(4)*dj43_c2);
        const T dj43_c4 = nt_div<T>(-D_coeb + dj43_c2, T(2)*(D_coea*D_coea));
        J[321] = (-d_D_argum_1*dj43_c3 + d_D_coeb_1*dj43_c1) * (cs1 * rs43);
        J[331] = (-d_D_argum_2*dj43_c3) * (cs2 * rs43);
        J[319] = (-d_D_argum_4*dj43_c3 + d_D_coeb_4*dj43_c1) * (cs4 * rs43);
        J[322] = (-d_D_argum_8*dj43_c3 + d_D_coea_8*dj43_c4 + d_D_coeb_8*dj43_c1) * (cs8 * rs43);
        J[330] = (-d_D_argum_12*dj43_c3 + d_D_coeb_12*dj43_c1) * (cs12 * rs43);
        J[323] = (-d_D_argum_14*dj43_c3 + d_D_coeb_14*dj43_c1) * (cs14 * rs43);
        J[326] = (-d_D_argum_16*dj43_c3 + d_D_coea_16*dj43_c4 + d_D_coeb_16*dj43_c1) * (cs16 * rs43);
        J[325] = (-d_D_argum_18*dj43_c3 + d_D_coeb_18*dj43_c1) * (cs18 * rs43);
        J[320] = (-d_D_argum_21*dj43_c3 + d_D_coeb_21*dj43_c1) * (cs21 * rs43);
        J[317] = (-d_D_argum_25*dj43_c3) * (cs25 * rs43);
        J[329] = (-d_D_argum_27*dj43_c3 + d_D_coea_27*dj43_c4 + d_D_coeb_27*dj43_c1) * (cs27 * rs43);
        J[328] = (-d_D_argum_28*dj43_c3 + d_D_coeb_28*dj43_c1) * (cs28 * rs43);
        J[316] = (-d_D_argum_29*dj43_c3 + d_D_coeb_29*dj43_c1) * (cs29 * rs43);
        J[318] = (-d_D_argum_42*dj43_c3) * (cs42 * rs43);
        J[337] = (-d_D_argum_43*dj43_c3 + d_D_coea_43*dj43_c4 + d_D_coeb_43*dj43_c1 + T(1)) * (cs43 * rs43);
        J[334] = (-d_D_argum_44*dj43_c3 + d_D_coea_44*dj43_c4 + d_D_coeb_44*dj43_c1) * (cs44 * rs43);
        J[333] = (-d_D_argum_45*dj43_c3 + d_D_coea_45*dj43_c4 + d_D_coeb_45*dj43_c1) * (cs45 * rs43);
        J[339] = (-d_D_argum_46*dj43_c3 + d_D_coea_46*dj43_c4 + d_D_coeb_46*dj43_c1) * (cs46 * rs43);
        J[338] = (-d_D_argum_47*dj43_c3 + d_D_coea_47*dj43_c4 + d_D_coeb_47*dj43_c1) * (cs47 * rs43);
        J[332] = (-d_D_argum_48*dj43_c3 + d_D_coeb_48*dj43_c1) * (cs48 * rs43);
        J[340] = (-d_D_argum_49*dj43_c3 + d_D_coea_49*dj43_c4 + d_D_coeb_49*dj43_c1) * (cs49 * rs43);
        J[336] = (-d_D_argum_50*dj43_c3 + d_D_coea_50*dj43_c4 + d_D_coeb_50*dj43_c1) * (cs50 * rs43);
        J[341] = (-d_D_argum_52*dj43_c3 + d_D_coea_52*dj43_c4 + d_D_coeb_52*dj43_c1) * (cs52 * rs43);
        J[335] = (-d_D_argum_53*dj43_c3 + d_D_coea_53*dj43_c4 + d_D_coeb_53*dj43_c1) * (cs53 * rs43);
        J[327] = (-d_D_argum_55*dj43_c3 + d_D_coea_55*dj43_c4 + d_D_coeb_55*dj43_c1) * (cs55 * rs43);
        J[324] = (-d_D_argum_56*dj43_c3) * (cs56 * rs43);
    }
}

// residual rows [0, 2, 3, 4, 5, 6, 7, 9, 10, 15, 16, 18, 21, 22, 26, 30, 32, 34, 37, 38, 40, 41, 44, 46, 47, 48, 49, 56] (day equations, FP64)
template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>
__device__ __forceinline__ void nt_residual_day_w2_1(const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {
    R[0] = -ck0[0] + x[0]*(F.dt*(tj[J_n2o] + x[42]*(K[K_b38] + K[K_b39])) + T(1));
    const T dr2_c0 = x[29]*x[43];
    R[2] = -F.dt*(F.h2*K[K_a19]*x[43] + F.parthcl*K[K_d11]*x[12]*x[43] + F.parthno3*K[K_b27]*x[43]*x[4] + K[K_a30]*x[16]*x[43] + K[K_a31]*(x[43]*x[43]) + K[K_c17a]*dr2_c0 + K[K_c17b]*dr2_c0 + K[K_c2]*x[1]*x[43] + K[K_c8]*x[27]*x[43] + x[47]*(K[K_a17]*x[43] + T(1.6e-12)*x[55])) - ck0[2] + x[2]*(F.dt*F.parth2o*(K[K_a1et]*x[42] + tj[J_h2o]) + T(1));
    R[3] = -T(2)*F.dt*K[K_b39]*x[0]*x[42] + F.dt*(F.rain_hno3*x[4] + T(2)*K[K_b6]*x[49]*x[51]) - ck0[3] + x[3];
    R[4] = -F.dt*(K[K_b22]*x[43]*x[48] + het[0]*x[13]*x[2] + het[1]*x[12]*x[13] + T(2)*het[2]*x[2]*x[5] + het[3]*x[12]*x[5] + het[5]*x[19]*x[2]) - ck0[4] + x[4]*(F.dt*(F.parthno3*(K[K_b27]*x[43] + tj[J_hno3]) + F.rain_hno3) + T(1));
    R[5] = -F.dt*K[K_b12]*x[48]*x[54] - ck0[5] + x[5]*(F.dt*(F.hnm*K[K_b32] + het[2]*x[2] + het[3]*x[12] + tj[J_n2o5]) + T(1));
    const T dr6_c0 = T(3)*x[42];
    R[6] = F.dt*F.rain_hcl*x[12] - F.dt*(x[30]*(K[K_d90]*dr6_c0 + T(3)*tj[J_cfc11]) + x[31]*(T(2)*K[K_d91]*x[42] + T(2)*tj[J_cfc12]) + x[32]*(K[K_d92]*dr6_c0 + T(3)*tj[J_cfc113]) + x[33]*(T(4)*K[K_d93]*x[42] + T(4)*tj[J_ccl4]) + x[34]*(T(3)*K[K_d94]*x[43] + T(3)*tj[J_ch3ccl3]) + x[35]*(K[K_d95]*x[43] + tj[J_ch3cl]) + x[36]*(K[K_d96]*x[42] + K[K_d97]*x[43] + tj[J_hcfc22]) + x[38]*(K[K_e52]*x[42] + tj[J_h1211])) - ck0[6] + x[6];
    R[9] = -F.dt*K[K_e5a]*x[52]*x[53] - ck0[9] + x[9]*(F.dt*tj[J_oclo] + T(1));
    R[10] = -ck0[10] + x[10];
    R[15] = -F.dt*(K[K_d37]*x[14]*x[44] + K[K_d62]*(x[52]*x[52]) + het[1]*x[12]*x[13] + het[4]*x[12]*x[14]) - ck0[15] + x[15]*(F.dt*tj[J_cl2] + T(1));
    R[16] = -F.dt*K[K_a27]*(x[47]*x[47]) - ck0[16] + x[16]*(F.dt*(F.rain_h2o2 + K[K_a30]*x[43] + tj[J_h2o2]) + T(1));
    R[18] = -F.dt*(K[K_c19]*x[27]*x[50] + K[K_e7]*x[47]*x[50]) - ck0[18] + x[18]*(F.dt*(F.parthbr*(K[K_e11]*x[43] + K[K_e9]*x[42] + tj[J_hbr]) + F.rain_hbr + het[7]*x[25] + het[8]*x[14]) + T(1));
    R[21] = -F.dt*K[K_b23]*x[47]*x[48] - ck0[21] + x[21]*(F.dt*(F.hnm*K[K_b24] + K[K_b28]*x[43] + tj[J_hno4]) + T(1));
    const T dr22_c0 = T(2)*x[52];
    const T dr22_c1 = T(3)*x[42];
    R[22] = F.dt*(x[44]*(F.h2*K[K_d6] + K[K_c10]*x[27] + K[K_d36]*x[48] + K[K_d37]*x[14] + K[K_d5]*x[1] + K[K_d7]*x[47]) + x[52]*(K[K_d31]*x[48] + K[K_d33]*x[47] + K[K_d60]*dr22_c0 + K[K_d62]*dr22_c0 + K[K_d9]*x[43] + K[K_e5a]*x[53] + K[K_e5c]*x[53])) - F.dt*(F.parthcl*x[12]*(K[K_d11]*x[43] + tj[J_hcl]) + tj[J_brcl]*x[26] + T(2)*tj[J_cl2]*x[15] + tj[J_clno2]*x[17] + tj[J_oclo]*x[9] + x[13]*(K[K_d32]*x[45] + tj[J_clono2_cl] + tj[J_clono2_clo]) + x[14]*(K[K_d34]*x[43] + K[K_d35]*x[45] + tj[J_hocl]) + x[24]*(T(2)*F.hnm*K[K_d61] + T(2)*tj[J_cl2o2]) + x[30]*(K[K_d90]*dr22_c1 + T(3)*tj[J_cfc11]) + x[31]*(T(2)*K[K_d91]*x[42] + T(2)*tj[J_cfc12]) + x[32]*(K[K_d92]*dr22_c1 + T(3)*tj[J_cfc113]) + x[33]*(T(4)*K[K_d93]*x[42] + T(4)*tj[J_ccl4]) + x[34]*(T(3)*K[K_d94]*x[43] + T(3)*tj[J_ch3ccl3]) + x[35]*(K[K_d95]*x[43] + tj[J_ch3cl]) + x[36]*(K[K_d96]*x[42] + K[K_d97]*x[43] + tj[J_hcfc22])) - ck0[22] + x[22];
    R[26] = -F.dt*(K[K_e5c]*x[52]*x[53] + het[6]*x[12]*x[25] + het[8]*x[14]*x[18]) - ck0[26] + x[26]*(F.dt*tj[J_brcl] + T(1));
    R[30] = -ck0[30] + x[30]*(F.dt*(K[K_d90]*x[42] + tj[J_cfc11]) + T(1));
    R[32] = -ck0[32] + x[32]*(F.dt*(K[K_d92]*x[42] + tj[J_cfc113]) + T(1));
    R[34] = -ck0[34] + x[34]*(F.dt*(K[K_d94]*x[43] + tj[J_ch3ccl3]) + T(1));
    R[37] = -ck0[37] + x[37]*(F.dt*(K[K_e50]*x[42] + K[K_e51]*x[43] + tj[J_ch3br]) + T(1));
    R[38] = -ck0[38] + x[38]*(F.dt*(K[K_e52]*x[42] + tj[J_h1211]) + T(1));
    R[40] = F.dt*F.rain_hbr*x[18] - F.dt*(x[37]*(K[K_e50]*x[42] + K[K_e51]*x[43] + tj[J_ch3br]) + x[38]*(K[K_e52]*x[42] + tj[J_h1211]) + x[39]*(K[K_e53]*x[42] + tj[J_h1301]) + x[41]*(T(2)*K[K_e54]*x[43] + T(2)*tj[J_ch2br2])) - ck0[40] + x[40];
    R[41] = -ck0[41] + x[41]*(F.dt*(K[K_e54]*x[43] + tj[J_ch2br2]) + T(1));
    R[56] = nt_div<T>(-x[1]*(K[K_c1a]*x[42] + K[K_c2]*x[43] + K[K_d5]*x[44]), F.o2*K[K_c4] + K[K_c3]*x[45]) + x[56];
    const T D_r1 = nt_div<T>(K[K_a2]*x[55] + K[K_a6]*x[43] + K[K_a6b]*x[47] + K[K_b4]*x[49] + K[K_d2]*x[44] + tj[J_o3_o1d] + tj[J_o3_o3p], F.o2*K[K_hk2]);
    R[46] = x[46] + nt_div<T>(-x[7], D_r1 + T(1));
    const T D_r4 = nt_div<T>(F.h2*K[K_a19] + K[K_a36]*x[8] + K[K_a5]*x[45], F.o2*K[K_a1] + K[K_a2]*x[46] + T(8.049999999999999e-11)*x[47]);
    const T D_r7 = nt_div<T>(tj[J_no], F.o2*K[K_b7] + K[K_b6]*x[49]);
    const T D_r8 = nt_div<T>(K[K_b9]*x[46], K[K_b12]*x[48] + tj[J_no3_no2] + tj[J_no3_no]);
    const T D_r5 = nt_div<T>(D_r8*tj[J_no3_no] + K[K_b3]*x[45] + tj[J_no2], K[K_a26]*x[47] + K[K_b4]*x[46] + K[K_c5]*x[28] + K[K_d4]*x[52] + K[K_e4]*x[53]);
    R[48] = nt_div<T>(-x[20], D_r5*D_r7 + D_r5 + D_r8 + T(1)) + x[48];
    R[49] = -D_r5*x[48] + x[49];
    const T D_r6 = nt_div<T>(D_r4*F.o2*K[K_a1] + K[K_a30]*x[16] + K[K_a6]*x[46] + K[K_c8]*x[27] + K[K_d8]*x[52] + K[K_e10]*x[53], K[K_a17]*x[43] + K[K_a26]*x[49] + T(2)*K[K_a27]*x[47] + K[K_a6b]*x[46] + K[K_a7]*x[45] + K[K_d10]*x[44] + K[K_d33]*x[52] + K[K_d7]*x[44] + K[K_e15]*x[53] + K[K_e7]*x[50] + T(8.049999999999999e-11)*x[55]);
    R[47] = -D_r6*x[43] + x[47];
    const T D_r13 = nt_div<T>(K[K_d31]*x[48], K[K_d32]*x[45] + het[0]*x[2] + het[1]*x[12] + tj[J_clono2_cl] + tj[J_clono2_clo]);
    const T D_r9 = nt_div<T>(D_r13*het[0]*x[2] + K[K_d33]*x[47], K[K_d35]*x[45] + het[4]*x[12] + tj[J_hocl]);
    const T D_r10 = nt_div<T>(K[K_d60]*x[52], F.hnm*K[K_d61] + tj[J_cl2o2]);
    const T D_r12 = nt_div<T>(K[K_e5c]*x[53], tj[J_brcl]);
    const T D_r11 = nt_div<T>(T(2)*D_r10*tj[J_cl2o2] + D_r12*tj[J_brcl] + D_r13*tj[J_clono2_cl] + D_r9*tj[J_hocl] + K[K_c18]*x[28] + K[K_d3]*x[45] + K[K_d4]*x[49] + K[K_d8]*x[43] + K[K_e5b]*x[53], K[K_d10]*x[47] + K[K_d2]*x[46] + K[K_d37]*x[14] + K[K_d5]*x[1] + K[K_d7]*x[47]);
    R[44] = -D_r11*x[52] + x[44];
    const T D_t06_c0 = tj[J_hocl]*x[14];
    const T D_t06_c1 = K[K_d33]*x[47]*x[52];
    const bool sel_D_t06 = (D_t06_c0) <= (D_t06_c1);
    const T D_t06 = sel_D_t06 ? T(D_t06_c0) : T(D_t06_c1);
    const T D_t07_c0 = K[K_e5c]*x[52]*x[53];
    const T D_t07_c1 = tj[J_brcl]*x[26];
    const bool sel_D_t07 = (D_t07_c0) <= (D_t07_c1);
    const T D_t07 = sel_D_t07 ? T(D_t07_c0) : T(D_t07_c1);
    const T D_t09_c0 = K[K_e15]*x[47]*x[53];
    const T D_t09_c1 = tj[J_hobr]*x[25];
    const bool sel_D_t09 = (D_t09_c0) <= (D_t09_c1);
    const T D_t09 = sel_D_t09 ? T(D_t09_c0) : T(D_t09_c1);
    const T dr7_c0 = T(2)*x[45];
    const T dr7_c1 = nt_div<T>(T(2)*tj[J_no3_no], fmax(T(1e-30), tj[J_no3_no2] + tj[J_no3_no]));
    R[7] = -F.dt*(T(2)*F.o2*tj[J_o2] + K[K_a26]*x[47]*x[49] + K[K_c5]*x[28]*x[49]) + F.dt*(D_t06 + T(2)*D_t07 + D_t09 + K[K_b3]*dr7_c0*x[48] + K[K_b9]*dr7_c1*x[46]*x[48] + K[K_d3]*dr7_c0*x[52] + nt_div<T>(T(2)*K[K_d60]*tj[J_cl2o2]*(x[52]*x[52]), F.hnm*K[K_d61] + tj[J_cl2o2]) + T(2)*K[K_e5b]*x[52]*x[53] + T(2)*K[K_e6]*(x[53]*x[53]) + T(2)*K[K_hk1]*(x[45]*x[45]) + K[K_hk3]*dr7_c0*x[46] + dr7_c1*tj[J_clono2_cl]*x[13] + x[45]*(K[K_a5]*x[43] + K[K_a7]*x[47]) + x[46]*(K[K_a2]*x[55] + K[K_a6]*x[43] + K[K_a6b]*x[47])) - ck0[7] + x[7];
}

// scaled Jacobian rows [0, 1, 3, 6, 7, 13, 19, 20, 21, 23, 24, 28, 31, 33, 35, 36, 39, 40, 42, 44, 45, 46, 47, 48, 50, 51, 52, 53, 54, 56] (day equations) into their stored A slots
template <typename T, typename FF, typename PK, typename PJ>
__device__ __forceinline__ void nt_jacobian_day_w2_1(const FF& F, PK K, PK tj, PK het, const double* __restrict__ x, double floor_, PJ J) {
    const int fh = nt_exp_hi(floor_);
    const T xt0 = nt_cvt<T>(x[0]);
    const T xt1 = nt_cvt<T>(x[1]);
    const T xt2 = nt_cvt<T>(x[2]);
    const T xt3 = nt_cvt<T>(x[3]);
    const T xt4 = nt_cvt<T>(x[4]);
    const T xt5 = nt_cvt<T>(x[5]);
    const T xt6 = nt_cvt<T>(x[6]);
    const T xt7 = nt_cvt<T>(x[7]);
    const T xt8 = nt_cvt<T>(x[8]);
    const T xt9 = nt_cvt<T>(x[9]);
    const T xt10 = nt_cvt<T>(x[10]);
    const T xt11 = nt_cvt<T>(x[11]);
    const T xt12 = nt_cvt<T>(x[12]);
    const T xt13 = nt_cvt<T>(x[13]);
    const T xt14 = nt_cvt<T>(x[14]);
    const T xt15 = nt_cvt<T>(x[15]);
    const T xt16 = nt_cvt<T>(x[16]);
    const T xt17 = nt_cvt<T>(x[17]);
    const T xt18 = nt_cvt<T>(x[18]);
    const T xt19 = nt_cvt<T>(x[19]);
    const T xt20 = nt_cvt<T>(x[20]);
    const T xt21 = nt_cvt<T>(x[21]);
    const T xt22 = nt_cvt<T>(x[22]);
    const T xt23 = nt_cvt<T>(x[23]);
    const T xt24 = nt_cvt<T>(x[24]);
    const T xt25 = nt_cvt<T>(x[25]);
    const T xt26 = nt_cvt<T>(x[26]);
    const T xt27 = nt_cvt<T>(x[27]);
    const T xt28 = nt_cvt<T>(x[28]);
    const T xt29 = nt_cvt<T>(x[29]);
    const T xt30 = nt_cvt<T>(x[30]);
    const T xt31 = nt_cvt<T>(x[31]);
    const T xt32 = nt_cvt<T>(x[32]);
    const T xt33 = nt_cvt<T>(x[33]);
    const T xt34 = nt_cvt<T>(x[34]);
    const T xt35 = nt_cvt<T>(x[35]);
    const T xt36 = nt_cvt<T>(x[36]);
    const T xt37 = nt_cvt<T>(x[37]);
    const T xt38 = nt_cvt<T>(x[38]);
    const T xt39 = nt_cvt<T>(x[39]);
    const T xt40 = nt_cvt<T>(x[40]);
    const T xt41 = nt_cvt<T>(x[41]);
    const T xt42 = nt_cvt<T>(x[42]);
    const T xt43 = nt_cvt<T>(x[43]);
    const T xt44 = nt_cvt<T>(x[44]);
    const T xt45 = nt_cvt<T>(x[45]);
    const T xt46 = nt_cvt<T>(x[46]);
    const T xt47 = nt_cvt<T>(x[47]);
    const T xt48 = nt_cvt<T>(x[48]);
    const T xt49 = nt_cvt<T>(x[49]);
    const T xt50 = nt_cvt<T>(x[50]);
    const T xt51 = nt_cvt<T>(x[51]);
    const T xt52 = nt_cvt<T>(x[52]);
    const T xt53 = nt_cvt<T>(x[53]);
    const T xt54 = nt_cvt<T>(x[54]);
    const T xt55 = nt_cvt<T>(x[55]);
    const T xt56 = nt_cvt<T>(x[56]);
    const T cs0 = nt_scale<T>(nt_exp_hi(x[0]), fh);
    const T cs1 = nt_scale<T>(nt_exp_hi(x[1]), fh);
    const T cs2 = nt_scale<T>(nt_exp_hi(x[2]), fh);
    const T cs4 = nt_scale<T>(nt_exp_hi(x[4]), fh);
    const T cs5 = nt_scale<T>(nt_exp_hi(x[5]), fh);
    const T cs7 = nt_scale<T>(nt_exp_hi(x[7]), fh);
    const T cs8 = nt_scale<T>(nt_exp_hi(x[8]), fh);
    const T cs12 = nt_scale<T>(nt_exp_hi(x[12]), fh);
    const T cs13 = nt_scale<T>(nt_exp_hi(x[13]), fh);
    const T cs14 = nt_scale<T>(nt_exp_hi(x[14]), fh);
    const T cs16 = nt_scale<T>(nt_exp_hi(x[16]), fh);
    const T cs17 = nt_scale<T>(nt_exp_hi(x[17]), fh);
    const T cs18 = nt_scale<T>(nt_exp_hi(x[18]), fh);
    const T cs19 = nt_scale<T>(nt_exp_hi(x[19]), fh);
    const T cs20 = nt_scale<T>(nt_exp_hi(x[20]), fh);
    const T cs21 = nt_scale<T>(nt_exp_hi(x[21]), fh);
    const T cs22 = nt_scale<T>(nt_exp_hi(x[22]), fh);
    const T cs23 = nt_scale<T>(nt_exp_hi(x[23]), fh);
    const T cs24 = nt_scale<T>(nt_exp_hi(x[24]), fh);
    const T cs25 = nt_scale<T>(nt_exp_hi(x[25]), fh);
    const T cs26 = nt_scale<T>(nt_exp_hi(x[26]), fh);
    const T cs27 = nt_scale<T>(nt_exp_hi(x[27]), fh);
    const T cs28 = nt_scale<T>(nt_exp_hi(x[28]), fh);
    const T cs29 = nt_scale<T>(nt_exp_hi(x[29]), fh);
    const T cs30 = nt_scale<T>(nt_exp_hi(x[30]), fh);
    const T cs31 = nt_scale<T>(nt_exp_hi(x[31]), fh);
    const T cs32 = nt_scale<T>(nt_exp_hi(x[32]), fh);
    const T cs33 = nt_scale<T>(nt_exp_hi(x[33]), fh);
    const T cs34 = nt_scale<T>(nt_exp_hi(x[34]), fh);
    const T cs35 = nt_scale<T>(nt_exp_hi(x[35]), fh);
    const T cs36 = nt_scale<T>(nt_exp_hi(x[36]), fh);
    const T cs37 = nt_scale<T>(nt_exp_hi(x[37]), fh);
    const T cs38 = nt_scale<T>(nt_exp_hi(x[38]), fh);
    const T cs39 = nt_scale<T>(nt_exp_hi(x[39]), fh);
    const T cs41 = nt_scale<T>(nt_exp_hi(x[41]), fh);
    const T cs42 = nt_scale<T>(nt_exp_hi(x[42]), fh);
    const T cs43 = nt_scale<T>(nt_exp_hi(x[43]), fh);
    const T cs44 = nt_scale<T>(nt_exp_hi(x[44]), fh);
    const T cs45 = nt_scale<T>(nt_exp_hi(x[45]), fh);
    const T cs46 = nt_scale<T>(nt_exp_hi(x[46]), fh);
    const T cs47 = nt_scale<T>(nt_exp_hi(x[47]), fh);
    const T cs48 = nt_scale<T>(nt_exp_hi(x[48]), fh);
    const T cs49 = nt_scale<T>(nt_exp_hi(x[49]), fh);
    const T cs50 = nt_scale<T>(nt_exp_hi(x[50]), fh);
    const T cs51 = nt_scale<T>(nt_exp_hi(x[51]), fh);
    const T cs52 = nt_scale<T>(nt_exp_hi(x[52]), fh);
    const T cs53 = nt_scale<T>(nt_exp_hi(x[53]), fh);
    const T cs54 = nt_scale<T>(nt_exp_hi(x[54]), fh);
    const T cs55 = nt_scale<T>(nt_exp_hi(x[55]), fh);
    const T cs56 = nt_scale<T>(nt_exp_hi(x[56]), fh);
    {  // row 0
    const T rs0 = nt_rscale<T>(nt_exp_hi(x[0]), fh);
        const T dj0_c0 = K[K_b38] + K[K_b39];
        J[76] = (F.dt*(dj0_c0*xt42 + tj[J_n2o]) + T(1)) * (cs0 * rs0);
        J[77] = (F.dt*dj0_c0*xt0) * (cs42 * rs0);
    }
    {  // row 1
    const T rs1 = nt_rscale<T>(nt_exp_hi(x[1]), fh);
        const T dj1_c0 = F.dt*xt1;
        J[157] = (F.dt*(K[K_c1a]*xt42 + K[K_c1b]*xt42 + K[K_c1c]*xt42 + K[K_c2]*xt43 + K[K_d5]*xt44) + T(1)) * (cs1 * rs1);
        J[156] = (dj1_c0*(K[K_c1a] + K[K_c1b] + K[K_c1c])) * (cs42 * rs1);
        J[159] = (K[K_c2]*dj1_c0) * (cs43 * rs1);
        J[158] = (K[K_d5]*dj1_c0) * (cs44 * rs1);
    }
    {  // row 3
    const T rs3 = nt_rscale<T>(nt_exp_hi(x[3]), fh);
        const T dj3_c0 = T(2)*F.dt;
        const T dj3_c1 = K[K_b39]*dj3_c0;
        const T dj3_c2 = K[K_b6]*dj3_c0;
        J[20] = (-dj3_c1*xt42) * (cs0 * rs3);
        J[23] = (F.dt*F.rain_hno3) * (cs4 * rs3);
        J[22] = (-dj3_c1*xt0) * (cs42 * rs3);
        J[24] = (dj3_c2*xt51) * (cs49 * rs3);
        J[21] = (dj3_c2*xt49) * (cs51 * rs3);
    }
    {  // row 6
    const T rs6 = nt_rscale<T>(nt_exp_hi(x[6]), fh);
        const T dj6_c0 = T(3)*xt42;
        const T dj6_c1 = T(2)*K[K_d91];
        const T dj6_c2 = T(4)*K[K_d93];
        const T dj6_c3 = T(3)*K[K_d94];
        J[9] = (F.dt*F.rain_hcl) * (cs12 * rs6);
        J[7] = (-F.dt*(K[K_d90]*dj6_c0 + T(3)*tj[J_cfc11])) * (cs30 * rs6);
        J[4] = (-F.dt*(dj6_c1*xt42 + T(2)*tj[J_cfc12])) * (cs31 * rs6);
        J[0] = (-F.dt*(K[K_d92]*dj6_c0 + T(3)*tj[J_cfc113])) * (cs32 * rs6);
        J[2] = (-F.dt*(dj6_c2*xt42 + T(4)*tj[J_ccl4])) * (cs33 * rs6);
        J[6] = (-F.dt*(dj6_c3*xt43 + T(3)*tj[J_ch3ccl3])) * (cs34 * rs6);
        J[5] = (-F.dt*(K[K_d95]*xt43 + tj[J_ch3cl])) * (cs35 * rs6);
        J[3] = (-F.dt*(K[K_d96]*xt42 + K[K_d97]*xt43 + tj[J_hcfc22])) * (cs36 * rs6);
        J[1] = (-F.dt*(K[K_e52]*xt42 + tj[J_h1211])) * (cs38 * rs6);
        J[8] = (-F.dt*(T(3)*K[K_d90]*xt30 + T(3)*K[K_d92]*xt32 + K[K_d96]*xt36 + K[K_e52]*xt38 + dj6_c1*xt31 + dj6_c2*xt33)) * (cs42 * rs6);
        J[10] = (-F.dt*(K[K_d95]*xt35 + K[K_d97]*xt36 + dj6_c3*xt34)) * (cs43 * rs6);
    }
    {  // row 13
    const T rs13 = nt_rscale<T>(nt_exp_hi(x[13]), fh);
        const T dj13_c0 = F.dt*xt13;
        const T dj13_c1 = F.dt*K[K_d31];
        J[89] = (dj13_c0*het[0]) * (cs2 * rs13);
        J[88] = (dj13_c0*het[1]) * (cs12 * rs13);
        J[87] = (F.dt*(K[K_d32]*xt45 + het[0]*xt2 + het[1]*xt12 + tj[J_clono2_cl] + tj[J_clono2_clo]) + T(1)) * (cs13 * rs13);
        J[91] = (K[K_d32]*dj13_c0) * (cs45 * rs13);
        J[90] = (-dj13_c1*xt52) * (cs48 * rs13);
        J[92] = (-dj13_c1*xt48) * (cs52 * rs13);
    }
    {  // row 19
    const T rs19 = nt_rscale<T>(nt_exp_hi(x[19]), fh);
        const T dj19_c0 = F.dt*xt19;
        const T dj19_c1 = F.dt*K[K_e13];
        J[56] = (dj19_c0*het[5]) * (cs2 * rs19);
        J[55] = (F.dt*(K[K_e8]*xt45 + het[5]*xt2 + tj[J_brono2]) + T(1)) * (cs19 * rs19);
        J[58] = (K[K_e8]*dj19_c0) * (cs45 * rs19);
        J[57] = (-dj19_c1*xt53) * (cs48 * rs19);
        J[59] = (-dj19_c1*xt48) * (cs53 * rs19);
    }
    {  // row 20
    const T rs20 = nt_rscale<T>(nt_exp_hi(x[20]), fh);
        const T dj20_c0 = T(2)*F.dt;
        const T dj20_c1 = K[K_b39]*dj20_c0;
        const T dj20_c2 = F.parthno3*K[K_b27];
        const T dj20_c3 = F.dt*xt48;
        const T dj20_c4 = T(2)*K[K_b12];
        const T dj20_c5 = K[K_b6]*dj20_c0;
        J[233] = (-dj20_c1*xt42) * (cs0 * rs20);
        J[237] = (-F.dt*(F.parthno3*tj[J_hno3] + dj20_c2*xt43)) * (cs4 * rs20);
        J[232] = (-F.dt*(T(2)*F.hnm*K[K_b32] + T(2)*tj[J_n2o5])) * (cs5 * rs20);
        J[235] = (-F.dt*(K[K_d32]*xt45 + tj[J_clono2_cl] + tj[J_clono2_clo])) * (cs13 * rs20);
        J[229] = (-F.dt*tj[J_clno2]) * (cs17 * rs20);
        J[230] = (-F.dt*(K[K_e8]*xt45 + tj[J_brono2])) * (cs19 * rs20);
        J[238] = (-F.dt*(F.hnm*K[K_b24] + K[K_b28]*xt43 + tj[J_hno4])) * (cs21 * rs20);
        J[236] = (-dj20_c1*xt0) * (cs42 * rs20);
        J[243] = (-F.dt*(K[K_b28]*xt21 + dj20_c2*xt4) + K[K_b22]*dj20_c3) * (cs43 * rs20);
        J[241] = (K[K_d36]*dj20_c3) * (cs44 * rs20);
        J[240] = (-F.dt*(K[K_d32]*xt13 + K[K_e8]*xt19)) * (cs45 * rs20);
        J[244] = (K[K_b23]*dj20_c3) * (cs47 * rs20);
        J[239] = (F.dt*(K[K_b22]*xt43 + K[K_b23]*xt47 + K[K_d31]*xt52 + K[K_d36]*xt44 + K[K_e13]*xt53 + dj20_c4*xt54)) * (cs48 * rs20);
        J[245] = (dj20_c5*xt51) * (cs49 * rs20);
        J[234] = (dj20_c5*xt49) * (cs51 * rs20);
        J[246] = (K[K_d31]*dj20_c3) * (cs52 * rs20);
        J[242] = (K[K_e13]*dj20_c3) * (cs53 * rs20);
        J[231] = (dj20_c3*dj20_c4) * (cs54 * rs20);
    }
    {  // row 21
    const T rs21 = nt_rscale<T>(nt_exp_hi(x[21]), fh);
        const T dj21_c0 = F.dt*K[K_b23];
        J[152] = (F.dt*(F.hnm*K[K_b24] + K[K_b28]*xt43 + tj[J_hno4]) + T(1)) * (cs21 * rs21);
        J[154] = (F.dt*K[K_b28]*xt21) * (cs43 * rs21);
        J[155] = (-dj21_c0*xt48) * (cs47 * rs21);
        J[153] = (-dj21_c0*xt47) * (cs48 * rs21);
    }
    {  // row 23
    const T rs23 = nt_rscale<T>(nt_exp_hi(x[23]), fh);
        const T dj23_c0 = T(2)*het[7];
        const T dj23_c1 = F.dt*F.parthbr*xt18;
        const T dj23_c2 = F.dt*xt53;
        J[196] = (-F.dt*(F.parthbr*(K[K_e11]*xt43 + K[K_e9]*xt42 + tj[J_hbr]) + dj23_c0*xt25)) * (cs18 * rs23);
        J[193] = (-F.dt*(K[K_e8]*xt45 + tj[J_brono2])) * (cs19 * rs23);
        J[194] = (-F.dt*(K[K_e16]*xt45 + dj23_c0*xt18 + tj[J_hobr])) * (cs25 * rs23);
        J[192] = (-F.dt*tj[J_brcl]) * (cs26 * rs23);
        J[197] = (F.dt*K[K_c19]*xt50) * (cs27 * rs23);
        J[195] = (-K[K_e9]*dj23_c1) * (cs42 * rs23);
        J[202] = (-K[K_e11]*dj23_c1) * (cs43 * rs23);
        J[199] = (-F.dt*(K[K_e16]*xt25 + K[K_e8]*xt19)) * (cs45 * rs23);
        J[203] = (F.dt*(K[K_e15]*xt53 + K[K_e7]*xt50)) * (cs47 * rs23);
        J[198] = (K[K_e13]*dj23_c2) * (cs48 * rs23);
        J[201] = (F.dt*(K[K_c19]*xt27 + K[K_e7]*xt47)) * (cs50 * rs23);
        J[204] = (K[K_e5c]*dj23_c2) * (cs52 * rs23);
        J[200] = (F.dt*(K[K_e13]*xt48 + K[K_e15]*xt47 + K[K_e5c]*xt52)) * (cs53 * rs23);
    }
    {  // row 24
    const T rs24 = nt_rscale<T>(nt_exp_hi(x[24]), fh);
        J[97] = (F.dt*(F.hnm*K[K_d61] + tj[J_cl2o2]) + T(1)) * (cs24 * rs24);
        J[98] = (-T(2)*F.dt*K[K_d60]*xt52) * (cs52 * rs24);
    }
    {  // row 28
    const T rs28 = nt_rscale<T>(nt_exp_hi(x[28]), fh);
        const T dj28_c0 = T(2)*K[K_c14]*xt28;
        const T dj28_c1 = F.dt*K[K_c17a];
        const T dj28_c2 = F.dt*xt28;
        J[212] = (F.dt*dj28_c0 + F.dt*(K[K_c18]*xt52 + K[K_c5]*xt49 + K[K_c7]*xt47 + dj28_c0) + T(1)) * (cs28 * rs28);
        J[210] = (-dj28_c1*xt43) * (cs29 * rs28);
        J[213] = (-dj28_c1*xt29) * (cs43 * rs28);
        J[214] = (K[K_c7]*dj28_c2) * (cs47 * rs28);
        J[215] = (K[K_c5]*dj28_c2) * (cs49 * rs28);
        J[216] = (K[K_c18]*dj28_c2) * (cs52 * rs28);
        J[211] = (-F.dt*F.o2*K[K_c4]) * (cs56 * rs28);
    }
    {  // row 31
    const T rs31 = nt_rscale<T>(nt_exp_hi(x[31]), fh);
        J[41] = (F.dt*(K[K_d91]*xt42 + tj[J_cfc12]) + T(1)) * (cs31 * rs31);
        J[42] = (F.dt*K[K_d91]*xt31) * (cs42 * rs31);
    }
    {  // row 33
    const T rs33 = nt_rscale<T>(nt_exp_hi(x[33]), fh);
        J[32] = (F.dt*(K[K_d93]*xt42 + tj[J_ccl4]) + T(1)) * (cs33 * rs33);
        J[33] = (F.dt*K[K_d93]*xt33) * (cs42 * rs33);
    }
    {  // row 35
    const T rs35 = nt_rscale<T>(nt_exp_hi(x[35]), fh);
        J[66] = (F.dt*(K[K_d95]*xt43 + tj[J_ch3cl]) + T(1)) * (cs35 * rs35);
        J[67] = (F.dt*K[K_d95]*xt35) * (cs43 * rs35);
    }
    {  // row 36
    const T rs36 = nt_rscale<T>(nt_exp_hi(x[36]), fh);
        const T dj36_c0 = F.dt*xt36;
        J[38] = (F.dt*(K[K_d96]*xt42 + K[K_d97]*xt43 + tj[J_hcfc22]) + T(1)) * (cs36 * rs36);
        J[39] = (K[K_d96]*dj36_c0) * (cs42 * rs36);
        J[40] = (K[K_d97]*dj36_c0) * (cs43 * rs36);
    }
    {  // row 39
    const T rs39 = nt_rscale<T>(nt_exp_hi(x[39]), fh);
        J[50] = (F.dt*(K[K_e53]*xt42 + tj[J_h1301]) + T(1)) * (cs39 * rs39);
        J[51] = (F.dt*K[K_e53]*xt39) * (cs42 * rs39);
    }
    {  // row 40
    const T rs40 = nt_rscale<T>(nt_exp_hi(x[40]), fh);
        const T dj40_c0 = T(2)*K[K_e54];
        J[16] = (F.dt*F.rain_hbr) * (cs18 * rs40);
        J[13] = (-F.dt*(K[K_e50]*xt42 + K[K_e51]*xt43 + tj[J_ch3br])) * (cs37 * rs40);
        J[11] = (-F.dt*(K[K_e52]*xt42 + tj[J_h1211])) * (cs38 * rs40);
        J[12] = (-F.dt*(K[K_e53]*xt42 + tj[J_h1301])) * (cs39 * rs40);
        J[15] = (-F.dt*(dj40_c0*xt43 + T(2)*tj[J_ch2br2])) * (cs41 * rs40);
        J[14] = (-F.dt*(K[K_e50]*xt37 + K[K_e52]*xt38 + K[K_e53]*xt39)) * (cs42 * rs40);
        J[17] = (-F.dt*(K[K_e51]*xt37 + dj40_c0*xt41)) * (cs43 * rs40);
    }
    {  // row 42
    const T rs42 = nt_rscale<T>(nt_exp_hi(x[42]), fh);
        J[99] = (nt_div<T>(-tj[J_o3_o1d], F.n2*K[K_hk4] + F.o2*K[K_hk5])) * (cs46 * rs42);
    }
    {  // row 56
    const T rs56 = nt_rscale<T>(nt_exp_hi(x[56]), fh);
        const T dj56_c0 = F.o2*K[K_c4] + K[K_c3]*xt45;
        const T dj56_c1 = nt_div<T>(T(1), dj56_c0);
        const T dj56_c2 = K[K_c1a]*xt42 + K[K_c2]*xt43 + K[K_d5]*xt44;
        const T dj56_c3 = dj56_c1*xt1;
        J[177] = (-dj56_c1*dj56_c2) * (cs1 * rs56);
        J[176] = (-K[K_c1a]*dj56_c3) * (cs42 * rs56);
        J[180] = (-K[K_c2]*dj56_c3) * (cs43 * rs56);
        J[179] = (-K[K_d5]*dj56_c3) * (cs44 * rs56);
        J[178] = (nt_div<T>(K[K_c3]*dj56_c2*xt1, (dj56_c0*dj56_c0))) * (cs45 * rs56);
    }
    const T D_r1_c0 = nt_div<T>(T(1), F.o2*K[K_hk2]);
    const T D_r1 = D_r1_c0*(K[K_a2]*xt55 + K[K_a6]*xt43 + K[K_a6b]*xt47 + K[K_b4]*xt49 + K[K_d2]*xt44 + tj[J_o3_o1d] + tj[J_o3_o3p]);
    const T d_D_r1_43 = D_r1_c0*K[K_a6];
    const T d_D_r1_44 = D_r1_c0*K[K_d2];
    const T d_D_r1_47 = D_r1_c0*K[K_a6b];
    const T d_D_r1_49 = D_r1_c0*K[K_b4];
    const T d_D_r1_55 = D_r1_c0*K[K_a2];
    {  // row 45
    const T rs45 = nt_rscale<T>(nt_exp_hi(x[45]), fh);
        J[280] = (-d_D_r1_43*xt46) * (cs43 * rs45);
        J[279] = (-d_D_r1_44*xt46) * (cs44 * rs45);
        J[282] = (-D_r1) * (cs46 * rs45);
        J[281] = (-d_D_r1_47*xt46) * (cs47 * rs45);
        J[283] = (-d_D_r1_49*xt46) * (cs49 * rs45);
        J[278] = (-d_D_r1_55*xt46) * (cs55 * rs45);
    }
    {  // row 46
    const T rs46 = nt_rscale<T>(nt_exp_hi(x[46]), fh);
        const T dj46_c0 = D_r1 + T(1);
        const T dj46_c1 = nt_div<T>(xt7, (dj46_c0*dj46_c0));
        J[355] = (nt_div<T>(T(-1), dj46_c0)) * (cs7 * rs46);
        J[358] = (d_D_r1_43*dj46_c1) * (cs43 * rs46);
        J[357] = (d_D_r1_44*dj46_c1) * (cs44 * rs46);
        J[359] = (d_D_r1_47*dj46_c1) * (cs47 * rs46);
        J[360] = (d_D_r1_49*dj46_c1) * (cs49 * rs46);
        J[356] = (d_D_r1_55*dj46_c1) * (cs55 * rs46);
    }
    const T D_r4_c0 = F.h2*K[K_a19] + K[K_a36]*xt8 + K[K_a5]*xt45;
    const T D_r4_c1 = F.o2*K[K_a1] + K[K_a2]*xt46 + T(8.049999999999999e-11)*xt47;
    const T D_r4_c2 = nt_div<T>(T(1), D_r4_c1);
    const T D_r4_c3 = nt_div<T>(D_r4_c0, (D_r4_c1*D_r4_c1));
    const T D_r4 = D_r4_c0*D_r4_c2;
    const T d_D_r4_8 = D_r4_c2*K[K_a36];
    const T d_D_r4_45 = D_r4_c2*K[K_a5];
    const T d_D_r4_46 = -D_r4_c3*K[K_a2];
    const T d_D_r4_47 = -T(8.049999999999999e-11)*D_r4_c3;
    const T D_r7_c0 = F.o2*K[K_b7] + K[K_b6]*xt49;
    const T D_r7 = nt_div<T>(tj[J_no], D_r7_c0);
    const T d_D_r7_49 = nt_div<T>(-K[K_b6]*tj[J_no], (D_r7_c0*D_r7_c0));
    {  // row 51
    const T rs51 = nt_rscale<T>(nt_exp_hi(x[51]), fh);
        J[78] = (-D_r7 - d_D_r7_49*xt49) * (cs49 * rs51);
    }
    const T D_r8_c0 = K[K_b12]*xt48 + tj[J_no3_no2] + tj[J_no3_no];
    const T D_r8_c1 = nt_div<T>(K[K_b9], D_r8_c0);
    const T D_r8 = D_r8_c1*xt46;
    const T d_D_r8_46 = D_r8_c1;
    const T d_D_r8_48 = nt_div<T>(-K[K_b12]*K[K_b9]*xt46, (D_r8_c0*D_r8_c0));
    {  // row 54
    const T rs54 = nt_rscale<T>(nt_exp_hi(x[54]), fh);
        J[68] = T(0);
        J[70] = (-d_D_r8_46*xt48) * (cs46 * rs54);
        J[69] = (-D_r8 - d_D_r8_48*xt48) * (cs48 * rs54);
    }
    const T D_r5_c0 = D_r8*tj[J_no3_no] + K[K_b3]*xt45 + tj[J_no2];
    const T D_r5_c1 = K[K_a26]*xt47 + K[K_b4]*xt46 + K[K_c5]*xt28 + K[K_d4]*xt52 + K[K_e4]*xt53;
    const T D_r5_c2 = nt_div<T>(T(1), D_r5_c1);
    const T D_r5_c3 = nt_div<T>(D_r5_c0, (D_r5_c1*D_r5_c1));
    const T D_r5 = D_r5_c0*D_r5_c2;
    const T d_D_r5_28 = -D_r5_c3*K[K_c5];
    const T d_D_r5_45 = D_r5_c2*K[K_b3];
    const T d_D_r5_46 = D_r5_c2*d_D_r8_46*tj[J_no3_no] - D_r5_c3*K[K_b4];
    const T d_D_r5_47 = -D_r5_c3*K[K_a26];
    const T d_D_r5_48 = D_r5_c2*d_D_r8_48*tj[J_no3_no];
    const T d_D_r5_52 = -D_r5_c3*K[K_d4];
    const T d_D_r5_53 = -D_r5_c3*K[K_e4];
    {  // row 48
    const T rs48 = nt_rscale<T>(nt_exp_hi(x[48]), fh);
        const T dj48_c0 = D_r5*D_r7 + D_r5 + D_r8 + T(1);
        const T dj48_c1 = nt_div<T>(T(1), dj48_c0*dj48_c0);
        const T dj48_c2 = dj48_c1*xt20;
        const T dj48_c3 = dj48_c2*(-D_r7 + T(-1));
        J[270] = (nt_div<T>(T(-1), dj48_c0)) * (cs20 * rs48);
        J[269] = (-d_D_r5_28*dj48_c3) * (cs28 * rs48);
        J[272] = (-d_D_r5_45*dj48_c3) * (cs45 * rs48);
        J[275] = (-d_D_r5_46*dj48_c3 + d_D_r8_46*dj48_c1*xt20) * (cs46 * rs48);
        J[274] = (-d_D_r5_47*dj48_c3) * (cs47 * rs48);
        J[271] = (-d_D_r5_48*dj48_c3 + d_D_r8_48*dj48_c2 + T(1)) * (cs48 * rs48);
        J[276] = (D_r5*d_D_r7_49*dj48_c2) * (cs49 * rs48);
        J[277] = (-d_D_r5_52*dj48_c3) * (cs52 * rs48);
        J[273] = (-d_D_r5_53*dj48_c3) * (cs53 * rs48);
    }
    const T D_r6_c0 = F.o2*K[K_a1];
    const T D_r6_c1 = D_r4*D_r6_c0 + K[K_a30]*xt16 + K[K_a6]*xt46 + K[K_c8]*xt27 + K[K_d8]*xt52 + K[K_e10]*xt53;
    const T D_r6_c2 = T(2)*K[K_a27];
    const T D_r6_c3 = D_r6_c2*xt47 + K[K_a17]*xt43 + K[K_a26]*xt49 + K[K_a6b]*xt46 + K[K_a7]*xt45 + K[K_d10]*xt44 + K[K_d33]*xt52 + K[K_d7]*xt44 + K[K_e15]*xt53 + K[K_e7]*xt50 + T(8.049999999999999e-11)*xt55;
    const T D_r6_c4 = nt_div<T>(T(1), D_r6_c3);
    const T D_r6_c5 = D_r6_c0*D_r6_c4;
    const T D_r6_c6 = nt_div<T>(D_r6_c1, (D_r6_c3*D_r6_c3));
    const T D_r6 = D_r6_c1*D_r6_c4;
    const T d_D_r6_8 = D_r6_c5*d_D_r4_8;
    const T d_D_r6_16 = D_r6_c4*K[K_a30];
    const T d_D_r6_27 = D_r6_c4*K[K_c8];
    const T d_D_r6_43 = -D_r6_c6*K[K_a17];
    const T d_D_r6_44 = D_r6_c6*(-K[K_d10] - K[K_d7]);
    const T d_D_r6_45 = D_r6_c5*d_D_r4_45 - D_r6_c6*K[K_a7];
    const T d_D_r6_46 = D_r6_c4*K[K_a6] + D_r6_c5*d_D_r4_46 - D_r6_c6*K[K_a6b];
    const T d_D_r6_47 = -D_r6_c2*D_r6_c6 + D_r6_c5*d_D_r4_47;
    const T d_D_r6_49 = -D_r6_c6*K[K_a26];
    const T d_D_r6_50 = -D_r6_c6*K[K_e7];
    const T d_D_r6_52 = D_r6_c4*K[K_d8] - D_r6_c6*K[K_d33];
    const T d_D_r6_53 = D_r6_c4*K[K_e10] - D_r6_c6*K[K_e15];
    const T d_D_r6_55 = -T(8.049999999999999e-11)*D_r6_c6;
    {  // row 47
    const T rs47 = nt_rscale<T>(nt_exp_hi(x[47]), fh);
        J[342] = (-d_D_r6_8*xt43) * (cs8 * rs47);
        J[343] = (-d_D_r6_16*xt43) * (cs16 * rs47);
        J[345] = (-d_D_r6_27*xt43) * (cs27 * rs47);
        J[350] = (-D_r6 - d_D_r6_43*xt43) * (cs43 * rs47);
        J[347] = (-d_D_r6_44*xt43) * (cs44 * rs47);
        J[346] = (-d_D_r6_45*xt43) * (cs45 * rs47);
        J[352] = (-d_D_r6_46*xt43) * (cs46 * rs47);
        J[351] = (-d_D_r6_47*xt43 + T(1)) * (cs47 * rs47);
        J[353] = (-d_D_r6_49*xt43) * (cs49 * rs47);
        J[349] = (-d_D_r6_50*xt43) * (cs50 * rs47);
        J[354] = (-d_D_r6_52*xt43) * (cs52 * rs47);
        J[348] = (-d_D_r6_53*xt43) * (cs53 * rs47);
        J[344] = (-d_D_r6_55*xt43) * (cs55 * rs47);
    }
    const T D_r13_c0 = K[K_d32]*xt45 + het[0]*xt2 + het[1]*xt12 + tj[J_clono2_cl] + tj[J_clono2_clo];
    const T D_r13_c1 = nt_div<T>(K[K_d31], D_r13_c0);
    const T D_r13_c2 = nt_div<T>(K[K_d31]*xt48, (D_r13_c0*D_r13_c0));
    const T D_r13 = D_r13_c1*xt48;
    const T d_D_r13_2 = -D_r13_c2*het[0];
    const T d_D_r13_12 = -D_r13_c2*het[1];
    const T d_D_r13_45 = -D_r13_c2*K[K_d32];
    const T d_D_r13_48 = D_r13_c1;
    const T D_r9_c0 = D_r13*het[0];
    const T D_r9_c1 = D_r9_c0*xt2 + K[K_d33]*xt47;
    const T D_r9_c2 = K[K_d35]*xt45 + het[4]*xt12 + tj[J_hocl];
    const T D_r9_c3 = nt_div<T>(T(1), D_r9_c2);
    const T D_r9_c4 = D_r9_c3*het[0]*xt2;
    const T D_r9_c5 = nt_div<T>(D_r9_c1, (D_r9_c2*D_r9_c2));
    const T D_r9 = D_r9_c1*D_r9_c3;
    const T d_D_r9_2 = D_r9_c0*D_r9_c3 + D_r9_c4*d_D_r13_2;
    const T d_D_r9_12 = D_r9_c4*d_D_r13_12 - D_r9_c5*het[4];
    const T d_D_r9_45 = D_r9_c3*d_D_r13_45*het[0]*xt2 - D_r9_c5*K[K_d35];
    const T d_D_r9_47 = D_r9_c3*K[K_d33];
    const T d_D_r9_48 = D_r9_c4*d_D_r13_48;
    const T D_r10_c0 = nt_div<T>(K[K_d60], F.hnm*K[K_d61] + tj[J_cl2o2]);
    const T D_r10 = D_r10_c0*xt52;
    const T d_D_r10_52 = D_r10_c0;
    const T D_r12_c0 = nt_div<T>(K[K_e5c], tj[J_brcl]);
    const T D_r12 = D_r12_c0*xt53;
    const T d_D_r12_53 = D_r12_c0;
    const T D_r11_c0 = K[K_d10]*xt47 + K[K_d2]*xt46 + K[K_d37]*xt14 + K[K_d5]*xt1 + K[K_d7]*xt47;
    const T D_r11_c1 = nt_div<T>(T(1), D_r11_c0);
    const T D_r11_c2 = T(2)*tj[J_cl2o2];
    const T D_r11_c3 = D_r10*D_r11_c2 + D_r12*tj[J_brcl] + D_r13*tj[J_clono2_cl] + D_r9*tj[J_hocl] + K[K_c18]*xt28 + K[K_d3]*xt45 + K[K_d4]*xt49 + K[K_d8]*xt43 + K[K_e5b]*xt53;
    const T D_r11_c4 = nt_div<T>(D_r11_c3, (D_r11_c0*D_r11_c0));
    const T D_r11_c5 = D_r11_c1*tj[J_clono2_cl];
    const T D_r11_c6 = D_r11_c1*tj[J_hocl];
    const T D_r11 = D_r11_c1*D_r11_c3;
    const T d_D_r11_1 = -D_r11_c4*K[K_d5];
    const T d_D_r11_2 = D_r11_c5*d_D_r13_2 + D_r11_c6*d_D_r9_2;
    const T d_D_r11_12 = D_r11_c5*d_D_r13_12 + D_r11_c6*d_D_r9_12;
    const T d_D_r11_14 = -D_r11_c4*K[K_d37];
    const T d_D_r11_28 = D_r11_c1*K[K_c18];
    const T d_D_r11_43 = D_r11_c1*K[K_d8];
    const T d_D_r11_45 = D_r11_c1*K[K_d3] + D_r11_c5*d_D_r13_45 + D_r11_c6*d_D_r9_45;
    const T d_D_r11_46 = -D_r11_c4*K[K_d2];
    const T d_D_r11_47 = D_r11_c4*(-K[K_d10] - K[K_d7]) + D_r11_c6*d_D_r9_47;
    const T d_D_r11_48 = D_r11_c5*d_D_r13_48 + D_r11_c6*d_D_r9_48;
    const T d_D_r11_49 = D_r11_c1*K[K_d4];
    const T d_D_r11_52 = D_r11_c1*D_r11_c2*d_D_r10_52;
    const T d_D_r11_53 = D_r11_c1*K[K_e5b] + D_r11_c1*d_D_r12_53*tj[J_brcl];
    {  // row 44
    const T rs44 = nt_rscale<T>(nt_exp_hi(x[44]), fh);
        J[284] = (-d_D_r11_1*xt52) * (cs1 * rs44);
        J[288] = (-d_D_r11_2*xt52) * (cs2 * rs44);
        J[287] = (-d_D_r11_12*xt52) * (cs12 * rs44);
        J[285] = (-d_D_r11_14*xt52) * (cs14 * rs44);
        J[286] = (-d_D_r11_28*xt52) * (cs28 * rs44);
        J[292] = (-d_D_r11_43*xt52) * (cs43 * rs44);
        J[290] = (-d_D_r11_45*xt52) * (cs45 * rs44);
        J[294] = (-d_D_r11_46*xt52) * (cs46 * rs44);
        J[293] = (-d_D_r11_47*xt52) * (cs47 * rs44);
        J[289] = (-d_D_r11_48*xt52) * (cs48 * rs44);
        J[295] = (-d_D_r11_49*xt52) * (cs49 * rs44);
        J[296] = (-D_r11 - d_D_r11_52*xt52) * (cs52 * rs44);
        J[291] = (-d_D_r11_53*xt52) * (cs53 * rs44);
    }
    {  // row 52
    const T rs52 = nt_rscale<T>(nt_exp_hi(x[52]), fh);
        const T dj52_c0 = D_r11 + T(1);
        const T dj52_c1 = nt_div<T>(xt22, (dj52_c0*dj52_c0));
        J[369] = (d_D_r11_1*dj52_c1) * (cs1 * rs52);
        J[373] = (d_D_r11_2*dj52_c1) * (cs2 * rs52);
        J[372] = (d_D_r11_12*dj52_c1) * (cs12 * rs52);
        J[370] = (d_D_r11_14*dj52_c1) * (cs14 * rs52);
        J[368] = (nt_div<T>(T(-1), dj52_c0)) * (cs22 * rs52);
        J[371] = (d_D_r11_28*dj52_c1) * (cs28 * rs52);
        J[377] = (d_D_r11_43*dj52_c1) * (cs43 * rs52);
        J[375] = (d_D_r11_45*dj52_c1) * (cs45 * rs52);
        J[379] = (d_D_r11_46*dj52_c1) * (cs46 * rs52);
        J[378] = (d_D_r11_47*dj52_c1) * (cs47 * rs52);
        J[374] = (d_D_r11_48*dj52_c1) * (cs48 * rs52);
        J[380] = (d_D_r11_49*dj52_c1) * (cs49 * rs52);
        J[381] = (d_D_r11_52*dj52_c1 + T(1)) * (cs52 * rs52);
        J[376] = (d_D_r11_53*dj52_c1) * (cs53 * rs52);
    }
    const T D_r27_c0 = K[K_e8]*xt45 + tj[J_brono2];
    const T D_r27_c1 = nt_div<T>(K[K_e13], D_r27_c0);
    const T D_r27 = D_r27_c1*xt48;
    const T d_D_r27_45 = nt_div<T>(-K[K_e13]*K[K_e8]*xt48, (D_r27_c0*D_r27_c0));
    const T d_D_r27_48 = D_r27_c1;
    const T D_r28_c0 = K[K_e16]*xt45 + tj[J_hobr];
    const T D_r28_c1 = nt_div<T>(K[K_e15], D_r28_c0);
    const T D_r28 = D_r28_c1*xt47;
    const T d_D_r28_45 = nt_div<T>(-K[K_e15]*K[K_e16]*xt47, (D_r28_c0*D_r28_c0));
    const T d_D_r28_47 = D_r28_c1;
    const T D_r29_c0 = nt_div<T>(K[K_e5c], tj[J_brcl]);
    const T D_r29 = D_r29_c0*xt52;
    const T d_D_r29_52 = D_r29_c0;
    const T D_r30_c0 = K[K_c19]*xt27 + K[K_e2]*xt46 + K[K_e7]*xt47;
    const T D_r30_c1 = nt_div<T>(T(1), D_r30_c0);
    const T D_r30_c2 = T(0.85)*tj[J_brono2];
    const T D_r30_c3 = T(2)*K[K_e6];
    const T D_r30_c4 = D_r27*D_r30_c2 + D_r28*tj[J_hobr] + D_r29*tj[J_brcl] + D_r30_c3*xt53 + K[K_e10]*xt43 + K[K_e3]*xt45 + K[K_e4]*xt49 + K[K_e5a]*xt52 + K[K_e5b]*xt52 + tj[J_bro];
    const T D_r30_c5 = nt_div<T>(D_r30_c4, (D_r30_c0*D_r30_c0));
    const T D_r30_c6 = D_r30_c1*D_r30_c2;
    const T D_r30 = D_r30_c1*D_r30_c4;
    const T d_D_r30_27 = -D_r30_c5*K[K_c19];
    const T d_D_r30_43 = D_r30_c1*K[K_e10];
    const T d_D_r30_45 = D_r30_c1*K[K_e3] + D_r30_c1*d_D_r28_45*tj[J_hobr] + D_r30_c6*d_D_r27_45;
    const T d_D_r30_46 = -D_r30_c5*K[K_e2];
    const T d_D_r30_47 = D_r30_c1*d_D_r28_47*tj[J_hobr] - D_r30_c5*K[K_e7];
    const T d_D_r30_48 = D_r30_c6*d_D_r27_48;
    const T d_D_r30_49 = D_r30_c1*K[K_e4];
    const T d_D_r30_52 = D_r30_c1*d_D_r29_52*tj[J_brcl] + D_r30_c1*(K[K_e5a] + K[K_e5b]);
    const T d_D_r30_53 = D_r30_c1*D_r30_c3;
    {  // row 50
    const T rs50 = nt_rscale<T>(nt_exp_hi(x[50]), fh);
        J[307] = (-d_D_r30_27*xt53) * (cs27 * rs50);
        J[311] = (-d_D_r30_43*xt53) * (cs43 * rs50);
        J[309] = (-d_D_r30_45*xt53) * (cs45 * rs50);
        J[313] = (-d_D_r30_46*xt53) * (cs46 * rs50);
        J[312] = (-d_D_r30_47*xt53) * (cs47 * rs50);
        J[308] = (-d_D_r30_48*xt53) * (cs48 * rs50);
        J[314] = (-d_D_r30_49*xt53) * (cs49 * rs50);
        J[315] = (-d_D_r30_52*xt53) * (cs52 * rs50);
        J[310] = (-D_r30 - d_D_r30_53*xt53) * (cs53 * rs50);
    }
    {  // row 53
    const T rs53 = nt_rscale<T>(nt_exp_hi(x[53]), fh);
        const T dj53_c0 = D_r30 + T(1);
        const T dj53_c1 = nt_div<T>(xt23, (dj53_c0*dj53_c0));
        J[297] = (nt_div<T>(T(-1), dj53_c0)) * (cs23 * rs53);
        J[298] = (d_D_r30_27*dj53_c1) * (cs27 * rs53);
        J[302] = (d_D_r30_43*dj53_c1) * (cs43 * rs53);
        J[300] = (d_D_r30_45*dj53_c1) * (cs45 * rs53);
        J[304] = (d_D_r30_46*dj53_c1) * (cs46 * rs53);
        J[303] = (d_D_r30_47*dj53_c1) * (cs47 * rs53);
        J[299] = (d_D_r30_48*dj53_c1) * (cs48 * rs53);
        J[305] = (d_D_r30_49*dj53_c1) * (cs49 * rs53);
        J[306] = (d_D_r30_52*dj53_c1) * (cs52 * rs53);
        J[301] = (d_D_r30_53*dj53_c1 + T(1)) * (cs53 * rs53);
    }
    const T D_t06_c0 = tj[J_hocl]*xt14;
    const T D_t06_c1 = K[K_d33]*xt52;
    const T D_t06_c2 = D_t06_c1*xt47;
    const bool sel_D_t06 = (D_t06_c0) <= (D_t06_c2);
    const T D_t06 = sel_D_t06 ? T(D_t06_c0) : T(D_t06_c2);
    const T d_D_t06_14 = sel_D_t06 ? T(tj[J_hocl]) : T(T(0));
    const T d_D_t06_47 = sel_D_t06 ? T(T(0)) : T(D_t06_c1);
    const T d_D_t06_52 = sel_D_t06 ? T(T(0)) : T(K[K_d33]*xt47);
    const T D_t07_c0 = K[K_e5c]*xt53;
    const T D_t07_c1 = D_t07_c0*xt52;
    const T D_t07_c2 = tj[J_brcl]*xt26;
    const bool sel_D_t07 = (D_t07_c1) <= (D_t07_c2);
    const T D_t07 = sel_D_t07 ? T(D_t07_c1) : T(D_t07_c2);
    const T d_D_t07_26 = sel_D_t07 ? T(T(0)) : T(tj[J_brcl]);
    const T d_D_t07_52 = sel_D_t07 ? T(D_t07_c0) : T(T(0));
    const T d_D_t07_53 = sel_D_t07 ? T(K[K_e5c]*xt52) : T(T(0));
    const T D_t09_c0 = K[K_e15]*xt53;
    const T D_t09_c1 = D_t09_c0*xt47;
    const T D_t09_c2 = tj[J_hobr]*xt25;
    const bool sel_D_t09 = (D_t09_c1) <= (D_t09_c2);
    const T D_t09 = sel_D_t09 ? T(D_t09_c1) : T(D_t09_c2);
    const T d_D_t09_25 = sel_D_t09 ? T(T(0)) : T(tj[J_hobr]);
    const T d_D_t09_47 = sel_D_t09 ? T(D_t09_c0) : T(T(0));
    const T d_D_t09_53 = sel_D_t09 ? T(K[K_e15]*xt47) : T(T(0));
    {  // row 7
    const T rs7 = nt_rscale<T>(nt_exp_hi(x[7]), fh);
        const T dj7_c0 = T(2)*F.dt;
        const T dj7_c1 = nt_div<T>(tj[J_no3_no], fmax(T(1e-30), tj[J_no3_no2] + tj[J_no3_no]));
        const T dj7_c2 = F.dt*xt49;
        const T dj7_c3 = T(2)*K[K_b3];
        const T dj7_c4 = T(2)*K[K_d3];
        const T dj7_c5 = T(2)*K[K_hk3];
        const T dj7_c6 = T(2)*K[K_b9]*dj7_c1;
        const T dj7_c7 = T(2)*K[K_e5b];
        J[105] = (dj7_c0*dj7_c1*tj[J_clono2_cl]) * (cs13 * rs7);
        J[106] = (F.dt*d_D_t06_14) * (cs14 * rs7);
        J[104] = (F.dt*d_D_t09_25) * (cs25 * rs7);
        J[103] = (d_D_t07_26*dj7_c0) * (cs26 * rs7);
        J[108] = (-K[K_c5]*dj7_c2) * (cs28 * rs7);
        J[112] = (F.dt*(K[K_a5]*xt45 + K[K_a6]*xt46)) * (cs43 * rs7);
        J[110] = (F.dt*(K[K_a5]*xt43 + K[K_a7]*xt47 + T(4)*K[K_hk1]*xt45 + dj7_c3*xt48 + dj7_c4*xt52 + dj7_c5*xt46)) * (cs45 * rs7);
        J[114] = (F.dt*(K[K_a2]*xt55 + K[K_a6]*xt43 + K[K_a6b]*xt47 + dj7_c5*xt45 + dj7_c6*xt48)) * (cs46 * rs7);
        J[113] = (F.dt*d_D_t06_47 + F.dt*d_D_t09_47 + F.dt*(K[K_a6b]*xt46 + K[K_a7]*xt45) - K[K_a26]*dj7_c2) * (cs47 * rs7);
        J[109] = (F.dt*(dj7_c3*xt45 + dj7_c6*xt46)) * (cs48 * rs7);
        J[115] = (-F.dt*(K[K_a26]*xt47 + K[K_c5]*xt28)) * (cs49 * rs7);
        J[116] = (F.dt*d_D_t06_52 + F.dt*(nt_div<T>(T(4)*K[K_d60]*tj[J_cl2o2]*xt52, F.hnm*K[K_d61] + tj[J_cl2o2]) + dj7_c4*xt45 + dj7_c7*xt53) + d_D_t07_52*dj7_c0) * (cs52 * rs7);
        J[111] = (F.dt*d_D_t09_53 + F.dt*(T(4)*K[K_e6]*xt53 + dj7_c7*xt52) + d_D_t07_53*dj7_c0) * (cs53 * rs7);
        J[107] = (F.dt*K[K_a2]*xt46) * (cs55 * rs7);
    }
}

// residual rows of group g of 2 (day equations)
template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>
__device__ __forceinline__ void nt_residual_day_w2(int g, const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {
    switch (g) {
        case 0: nt_residual_day_w2_0<T>(F, K, tj, het, ck0, x, R); break;
        case 1: nt_residual_day_w2_1<T>(F, K, tj, het, ck0, x, R); break;
        default: break;
    }
}
// Jacobian rows of group g of 2 (day equations)
template <typename T, typename FF, typename PK, typename PJ>
__device__ __forceinline__ void nt_jacobian_day_w2(int g, const FF& F, PK K, PK tj, PK het, const double* __restrict__ x, double floor_, PJ J) {
    switch (g) {
        case 0: nt_jacobian_day_w2_0<T>(F, K, tj, het, x, floor_, J); break;
        case 1: nt_jacobian_day_w2_1<T>(F, K, tj, het, x, floor_, J); break;
        default: break;
    }
}

// residual rows [5, 12, 14, 15, 21, 30, 34, 37, 41, 43, 55, 56] (day equations, FP64)
template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>
__device__ __forceinline__ void nt_residual_day_w4_0(const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {
    R[5] = -F.dt*K[K_b12]*x[48]*x[54] - ck0[5] + x[5]*(F.dt*(F.hnm*K[K_b32] + het[2]*x[2] + het[3]*x[12] + tj[J_n2o5]) + T(1));
    R[12] = -F.dt*(K[K_d9]*x[43]*x[52] + x[44]*(F.h2*K[K_d6] + K[K_c10]*x[27] + K[K_d5]*x[1] + K[K_d7]*x[47])) - ck0[12] + x[12]*(F.dt*(F.parthcl*(K[K_d11]*x[43] + tj[J_hcl]) + F.rain_hcl + het[1]*x[13] + het[3]*x[5] + het[4]*x[14] + het[6]*x[25]) + T(1));
    R[14] = -F.dt*(K[K_d33]*x[47]*x[52] + het[0]*x[13]*x[2]) - ck0[14] + x[14]*(F.dt*(K[K_d34]*x[43] + K[K_d35]*x[45] + K[K_d37]*x[44] + het[4]*x[12] + het[8]*x[18] + tj[J_hocl]) + T(1));
    R[15] = -F.dt*(K[K_d37]*x[14]*x[44] + K[K_d62]*(x[52]*x[52]) + het[1]*x[12]*x[13] + het[4]*x[12]*x[14]) - ck0[15] + x[15]*(F.dt*tj[J_cl2] + T(1));
    R[21] = -F.dt*K[K_b23]*x[47]*x[48] - ck0[21] + x[21]*(F.dt*(F.hnm*K[K_b24] + K[K_b28]*x[43] + tj[J_hno4]) + T(1));
    R[30] = -ck0[30] + x[30]*(F.dt*(K[K_d90]*x[42] + tj[J_cfc11]) + T(1));
    R[34] = -ck0[34] + x[34]*(F.dt*(K[K_d94]*x[43] + tj[J_ch3ccl3]) + T(1));
    R[37] = -ck0[37] + x[37]*(F.dt*(K[K_e50]*x[42] + K[K_e51]*x[43] + tj[J_ch3br]) + T(1));
    R[41] = -ck0[41] + x[41]*(F.dt*(K[K_e54]*x[43] + tj[J_ch2br2]) + T(1));
    R[56] = nt_div<T>(-x[1]*(K[K_c1a]*x[42] + K[K_c2]*x[43] + K[K_d5]*x[44]), F.o2*K[K_c4] + K[K_c3]*x[45]) + x[56];
    const T D_ch3o = nt_div<T>(K[K_c1b]*x[1]*x[42] + tj[J_ch3o2h]*x[29] + x[28]*(T(2)*K[K_c14]*x[28] + K[K_c18]*x[52] + K[K_c5]*x[49]), F.o2*K[K_c15]);
    const T D_hco = nt_div<T>(x[27]*(K[K_c10]*x[44] + K[K_c19]*x[50] + K[K_c8]*x[43] + K[K_c9]*x[45] + tj[J_ch2o_hco]), F.o2*K[K_c12]);
    const T D_r4 = nt_div<T>(F.h2*K[K_a19] + K[K_a36]*x[8] + K[K_a5]*x[45], F.o2*K[K_a1] + K[K_a2]*x[46] + T(8.049999999999999e-11)*x[47]);
    R[55] = -D_r4*x[43] + x[55];
    const T D_r6 = nt_div<T>(D_r4*F.o2*K[K_a1] + K[K_a30]*x[16] + K[K_a6]*x[46] + K[K_c8]*x[27] + K[K_d8]*x[52] + K[K_e10]*x[53], K[K_a17]*x[43] + K[K_a26]*x[49] + T(2)*K[K_a27]*x[47] + K[K_a6b]*x[46] + K[K_a7]*x[45] + K[K_d10]*x[44] + K[K_d33]*x[52] + K[K_d7]*x[44] + K[K_e15]*x[53] + K[K_e7]*x[50] + T(8.049999999999999e-11)*x[55]);
    const T D_coea = D_r6*(T(1.7e-11)*D_r4 + T(2)*D_r6*K[K_a27] + T(2)*K[K_a17]) + T(2)*K[K_a31];
    const T D_coeb = D_r6*K[K_b23]*x[48] + D_r6*K[K_c7]*x[28] + D_r6*K[K_d33]*x[52] + D_r6*K[K_d7]*x[44] + D_r6*K[K_e15]*x[53] + D_r6*K[K_e7]*x[50] + F.parthbr*K[K_e11]*x[18] + F.parthcl*K[K_d11]*x[12] + F.parthno3*K[K_b27]*x[4] + K[K_b22]*x[48] + K[K_b28]*x[21] + K[K_c17a]*x[29] + K[K_c2]*x[1] + K[K_c8]*x[27] + K[K_d34]*x[14] + K[K_d9]*x[52];
    const T D_coec = D_ch3o*F.o2*K[K_c15] + D_hco*F.o2*K[K_c12] + F.h2*K[K_d6]*x[44] + F.parth2o*x[2]*(T(2)*K[K_a1et]*x[42] + T(2)*tj[J_h2o]) + F.parthno3*tj[J_hno3]*x[4] + K[K_c3]*x[45]*x[56] + K[K_e16]*x[25]*x[45] + tj[J_ch3o2h]*x[29] + T(2)*tj[J_h2o2]*x[16] + tj[J_hbr]*x[18] + tj[J_hobr]*x[25] + x[14]*(K[K_d35]*x[45] + K[K_d37]*x[44] + tj[J_hocl]) + x[21]*(F.hnm*K[K_b24] + tj[J_hno4]) + x[27]*(K[K_c9]*x[45] + tj[J_ch2o_hco]) + x[42]*(T(2.4e-10)*F.h2 + x[1]*(K[K_c1a] + K[K_c1b]));
    const T D_argum_c0 = T(4)*D_coea*D_coec + (D_coeb*D_coeb);
    const bool sel_D_argum = (D_argum_c0) >= (T(0));
    const T D_argum = sel_D_argum ? T(D_argum_c0) : T(T(0));
    R[43] = x[43] + nt_div<T>(-(sqrt(D_argum) - D_coeb), T(2)*D_coea);
}

// scaled Jacobian rows [43] (day equations) into their stored A slots
template <typename T, typename FF, typename PK, typename PJ>
__device__ __forceinline__ void nt_jacobian_day_w4_0(const FF& F, PK K, PK tj, PK het, const double* __restrict__ x, double floor_, PJ J) {
    const int fh = nt_exp_hi(floor_);
    const T xt0 = nt_cvt<T>(x[0]);
    const T xt1 = nt_cvt<T>(x[1]);
    const T xt2 = nt_cvt<T>(x[2]);
    const T xt3 = nt_cvt<T>(x[3]);
    const T xt4 = nt_cvt<T>(x[4]);
    const T xt5 = nt_cvt<T>(x[5]);
    const T xt6 = nt_cvt<T>(x[6]);
    const T xt7 = nt_cvt<T>(x[7]);
    const T xt8 = nt_cvt<T>(x[8]);
    const T xt9 = nt_cvt<T>(x[9]);
    const T xt10 = nt_cvt<T>(x[10]);
    const T xt11 = nt_cvt<T>(x[11]);
    const T xt12 = nt_cvt<T>(x[12]);
    const T xt13 = nt_cvt<T>(x[13]);
    const T xt14 = nt_cvt<T>(x[14]);
    const T xt15 = nt_cvt<T>(x[15]);
    const T xt16 = nt_cvt<T>(x[16]);
    const T xt17 = nt_cvt<T>(x[17]);
    const T xt18 = nt_cvt<T>(x[18]);
    const T xt19 = nt_cvt<T>(x[19]);
    const T xt20 = nt_cvt<T>(x[20]);
    const T xt21 = nt_cvt<T>(x[21]);
    const T xt22 = nt_cvt<T>(x[22]);
    const T xt23 = nt_cvt<T>(x[23]);
    const T xt24 = nt_cvt<T>(x[24]);
    const T xt25 = nt_cvt<T>(x[25]);
    const T xt26 = nt_cvt<T>(x[26]);
    const T xt27 = nt_cvt<T>(x[27]);
    const T xt28 = nt_cvt<T>(x[28]);
    const T xt29 = nt_cvt<T>(x[29]);
    const T xt30 = nt_cvt<T>(x[30]);
    const T xt31 = nt_cvt<T>(x[31]);
    const T xt32 = nt_cvt<T>(x[32]);
    const T xt33 = nt_cvt<T>(x[33]);
    const T xt34 = nt_cvt<T>(x[34]);
    const T xt35 = nt_cvt<T>(x[35]);
    const T xt36 = nt_cvt<T>(x[36]);
    const T xt37 = nt_cvt<T>(x[37]);
    const T xt38 = nt_cvt<T>(x[38]);
    const T xt39 = nt_cvt<T>(x[39]);
    const T xt40 = nt_cvt<T>(x[40]);
    const T xt41 = nt_cvt<T>(x[41]);
    const T xt42 = nt_cvt<T>(x[42]);
    const T xt43 = nt_cvt<T>(x[43]);
    const T xt44 = nt_cvt<T>(x[44]);
    const T xt45 = nt_cvt<T>(x[45]);
    const T xt46 = nt_cvt<T>(x[46]);
    const T xt47 = nt_cvt<T>(x[47]);
    const T xt48 = nt_cvt<T>(x[48]);
    const T xt49 = nt_cvt<T>(x[49]);
    const T xt50 = nt_cvt<T>(x[50]);
    const T xt51 = nt_cvt<T>(x[51]);
    const T xt52 = nt_cvt<T>(x[52]);
    const T xt53 = nt_cvt<T>(x[53]);
    const T xt54 = nt_cvt<T>(x[54]);
    const T xt55 = nt_cvt<T>(x[55]);
    const T xt56 = nt_cvt<T>(x[56]);
    const T cs1 = nt_scale<T>(nt_exp_hi(x[1]), fh);
    const T cs2 = nt_scale<T>(nt_exp_hi(x[2]), fh);
    const T cs4 = nt_scale<T>(nt_exp_hi(x[4]), fh);
    const T cs8 = nt_scale<T>(nt_exp_hi(x[8]), fh);
    const T cs12 = nt_scale<T>(nt_exp_hi(x[12]), fh);
    const T cs14 = nt_scale<T>(nt_exp_hi(x[14]), fh);
    const T cs16 = nt_scale<T>(nt_exp_hi(x[16]), fh);
    const T cs18 = nt_scale<T>(nt_exp_hi(x[18]), fh);
    const T cs21 = nt_scale<T>(nt_exp_hi(x[21]), fh);
    const T cs25 = nt_scale<T>(nt_exp_hi(x[25]), fh);
    const T cs27 = nt_scale<T>(nt_exp_hi(x[27]), fh);
    const T cs28 = nt_scale<T>(nt_exp_hi(x[28]), fh);
    const T cs29 = nt_scale<T>(nt_exp_hi(x[29]), fh);
    const T cs42 = nt_scale<T>(nt_exp_hi(x[42]), fh);
    const T cs43 = nt_scale<T>(nt_exp_hi(x[43]), fh);
    const T cs44 = nt_scale<T>(nt_exp_hi(x[44]), fh);
    const T cs45 = nt_scale<T>(nt_exp_hi(x[45]), fh);
    const T cs46 = nt_scale<T>(nt_exp_hi(x[46]), fh);
    const T cs47 = nt_scale<T>(nt_exp_hi(x[47]), fh);
    const T cs48 = nt_scale<T>(nt_exp_hi(x[48]), fh);
    const T cs49 = nt_scale<T>(nt_exp_hi(x[49]), fh);
    const T cs50 = nt_scale<T>(nt_exp_hi(x[50]), fh);
    const T cs52 = nt_scale<T>(nt_exp_hi(x[52]), fh);
    const T cs53 = nt_scale<T>(nt_exp_hi(x[53]), fh);
    const T cs55 = nt_scale<T>(nt_exp_hi(x[55]), fh);
    const T cs56 = nt_scale<T>(nt_exp_hi(x[56]), fh);
    const T D_ch3o_c0 = K[K_c1b]*xt42;
    const T D_ch3o_c1 = K[K_c14]*xt28;
    const T D_ch3o_c2 = K[K_c18]*xt52 + K[K_c5]*xt49;
    const T D_ch3o_c3 = nt_div<T>(T(1), F.o2*K[K_c15]);
    const T D_ch3o_c4 = D_ch3o_c3*xt28;
    const T D_ch3o = D_ch3o_c3*(D_ch3o_c0*xt1 + tj[J_ch3o2h]*xt29 + xt28*(T(2)*D_ch3o_c1 + D_ch3o_c2));
    const T d_D_ch3o_1 = D_ch3o_c0*D_ch3o_c3;
    const T d_D_ch3o_28 = D_ch3o_c3*(T(4)*D_ch3o_c1 + D_ch3o_c2);
    const T d_D_ch3o_29 = D_ch3o_c3*tj[J_ch3o2h];
    const T d_D_ch3o_42 = D_ch3o_c3*K[K_c1b]*xt1;
    const T d_D_ch3o_49 = D_ch3o_c4*K[K_c5];
    const T d_D_ch3o_52 = D_ch3o_c4*K[K_c18];
    const T D_hco_c0 = nt_div<T>(T(1), F.o2*K[K_c12]);
    const T D_hco_c1 = D_hco_c0*(K[K_c10]*xt44 + K[K_c19]*xt50 + K[K_c8]*xt43 + K[K_c9]*xt45 + tj[J_ch2o_hco]);
    const T D_hco_c2 = D_hco_c0*xt27;
    const T D_hco = D_hco_c1*xt27;
    const T d_D_hco_27 = D_hco_c1;
    const T d_D_hco_43 = D_hco_c2*K[K_c8];
    const T d_D_hco_44 = D_hco_c2*K[K_c10];
    const T d_D_hco_45 = D_hco_c2*K[K_c9];
    const T d_D_hco_50 = D_hco_c2*K[K_c19];
    const T D_r4_c0 = F.h2*K[K_a19] + K[K_a36]*xt8 + K[K_a5]*xt45;
    const T D_r4_c1 = F.o2*K[K_a1] + K[K_a2]*xt46 + T(8.049999999999999e-11)*xt47;
    const T D_r4_c2 = nt_div<T>(T(1), D_r4_c1);
    const T D_r4_c3 = nt_div<T>(D_r4_c0, (D_r4_c1*D_r4_c1));
    const T D_r4 = D_r4_c0*D_r4_c2;
    const T d_D_r4_8 = D_r4_c2*K[K_a36];
    const T d_D_r4_45 = D_r4_c2*K[K_a5];
    const T d_D_r4_46 = -D_r4_c3*K[K_a2];
    const T d_D_r4_47 = -T(8.049999999999999e-11)*D_r4_c3;
    const T D_r6_c0 = F.o2*K[K_a1];
    const T D_r6_c1 = D_r4*D_r6_c0 + K[K_a30]*xt16 + K[K_a6]*xt46 + K[K_c8]*xt27 + K[K_d8]*xt52 + K[K_e10]*xt53;
    const T D_r6_c2 = T(2)*K[K_a27];
    const T D_r6_c3 = D_r6_c2*xt47 + K[K_a17]*xt43 + K[K_a26]*xt49 + K[K_a6b]*xt46 + K[K_a7]*xt45 + K[K_d10]*xt44 + K[K_d33]*xt52 + K[K_d7]*xt44 + K[K_e15]*xt53 + K[K_e7]*xt50 + T(8.049999999999999e-11)*xt55;
    const T D_r6_c4 = nt_div<T>(T(1), D_r6_c3);
    const T D_r6_c5 = D_r6_c0*D_r6_c4;
    const T D_r6_c6 = nt_div<T>(D_r6_c1, (D_r6_c3*D_r6_c3));
    const T D_r6 = D_r6_c1*D_r6_c4;
    const T d_D_r6_8 = D_r6_c5*d_D_r4_8;
    const T d_D_r6_16 = D_r6_c4*K[K_a30];
    const T d_D_r6_27 = D_r6_c4*K[K_c8];
    const T d_D_r6_43 = -D_r6_c6*K[K_a17];
    const T d_D_r6_44 = D_r6_c6*(-K[K_d10] - K[K_d7]);
    const T d_D_r6_45 = D_r6_c5*d_D_r4_45 - D_r6_c6*K[K_a7];
    const T d_D_r6_46 = D_r6_c4*K[K_a6] + D_r6_c5*d_D_r4_46 - D_r6_c6*K[K_a6b];
    const T d_D_r6_47 = -D_r6_c2*D_r6_c6 + D_r6_c5*d_D_r4_47;
    const T d_D_r6_49 = -D_r6_c6*K[K_a26];
    const T d_D_r6_50 = -D_r6_c6*K[K_e7];
    const T d_D_r6_52 = D_r6_c4*K[K_d8] - D_r6_c6*K[K_d33];
    const T d_D_r6_53 = D_r6_c4*K[K_e10] - D_r6_c6*K[K_e15];
    const T d_D_r6_55 = -T(8.049999999999999e-11)*D_r6_c6;
    const T D_coea_c0 = D_r6*K[K_a27];
    const T D_coea_c1 = T(1.7e-11)*D_r4 + T(2)*K[K_a17];
    const T D_coea_c2 = T(1.7e-11)*D_r6;
    const T D_coea_c3 = T(4)*D_coea_c0 + D_coea_c1;
    const T D_coea = D_r6*(T(2)*D_coea_c0 + D_coea_c1) + T(2)*K[K_a31];
    const T d_D_coea_8 = D_coea_c2*d_D_r4_8 + D_coea_c3*d_D_r6_8;
    const T d_D_coea_16 = D_coea_c3*d_D_r6_16;
    const T d_D_coea_27 = D_coea_c3*d_D_r6_27;
    const T d_D_coea_43 = D_coea_c3*d_D_r6_43;
    const T d_D_coea_44 = D_coea_c3*d_D_r6_44;
    const T d_D_coea_45 = D_coea_c2*d_D_r4_45 + D_coea_c3*d_D_r6_45;
    const T d_D_coea_46 = D_coea_c2*d_D_r4_46 + D_coea_c3*d_D_r6_46;
    const T d_D_coea_47 = D_coea_c2*d_D_r4_47 + D_coea_c3*d_D_r6_47;
    const T d_D_coea_49 = D_coea_c3*d_D_r6_49;
    const T d_D_coea_50 = D_coea_c3*d_D_r6_50;
    const T d_D_coea_52 = D_coea_c3*d_D_r6_52;
    const T d_D_coea_53 = D_coea_c3*d_D_r6_53;
    const T d_D_coea_55 = D_coea_c3*d_D_r6_55;
    const T D_coeb_c0 = K[K_b23]*xt48;
    const T D_coeb_c1 = K[K_c7]*xt28;
    const T D_coeb_c2 = K[K_d33]*xt52;
    const T D_coeb_c3 = K[K_d7]*xt44;
    const T D_coeb_c4 = K[K_e15]*xt53;
    const T D_coeb_c5 = K[K_e7]*xt50;
    const T D_coeb_c6 = F.parthbr*K[K_e11];
    const T D_coeb_c7 = F.parthcl*K[K_d11];
    const T D_coeb_c8 = F.parthno3*K[K_b27];
    const T D_coeb_c9 = D_coeb_c0 + D_coeb_c1 + D_coeb_c2 + D_coeb_c3 + D_coeb_c4 + D_coeb_c5;
    const T D_coeb = D_coeb_c0*D_r6 + D_coeb_c1*D_r6 + D_coeb_c2*D_r6 + D_coeb_c3*D_r6 + D_coeb_c4*D_r6 + D_coeb_c5*D_r6 + D_coeb_c6*xt18 + D_coeb_c7*xt12 + D_coeb_c8*xt4 + K[K_b22]*xt48 + K[K_b28]*xt21 + K[K_c17a]*xt29 + K[K_c2]*xt1 + K[K_c8]*xt27 + K[K_d34]*xt14 + K[K_d9]*xt52;
    const T d_D_coeb_1 = K[K_c2];
    const T d_D_coeb_4 = D_coeb_c8;
    const T d_D_coeb_8 = D_coeb_c9*d_D_r6_8;
    const T d_D_coeb_12 = D_coeb_c7;
    const T d_D_coeb_14 = K[K_d34];
    const T d_D_coeb_16 = D_coeb_c9*d_D_r6_16;
    const T d_D_coeb_18 = D_coeb_c6;
    const T d_D_coeb_21 = K[K_b28];
    const T d_D_coeb_27 = D_coeb_c9*d_D_r6_27 + K[K_c8];
    const T d_D_coeb_28 = D_r6*K[K_c7];
    const T d_D_coeb_29 = K[K_c17a];
    const T d_D_coeb_43 = D_coeb_c9*d_D_r6_43;
    const T d_D_coeb_44 = D_coeb_c9*d_D_r6_44 + D_r6*K[K_d7];
    const T d_D_coeb_45 = D_coeb_c9*d_D_r6_45;
    const T d_D_coeb_46 = D_coeb_c9*d_D_r6_46;
    const T d_D_coeb_47 = D_coeb_c9*d_D_r6_47;
    const T d_D_coeb_48 = D_r6*K[K_b23] + K[K_b22];
    const T d_D_coeb_49 = D_coeb_c9*d_D_r6_49;
    const T d_D_coeb_50 = D_coeb_c9*d_D_r6_50 + D_r6*K[K_e7];
    const T d_D_coeb_52 = D_coeb_c9*d_D_r6_52 + D_r6*K[K_d33] + K[K_d9];
    const T d_D_coeb_53 = D_coeb_c9*d_D_r6_53 + D_r6*K[K_e15];
    const T d_D_coeb_55 = D_coeb_c9*d_D_r6_55;
    const T D_coec_c0 = T(2)*tj[J_h2o2];
    const T D_coec_c1 = F.o2*K[K_c15];
    const T D_coec_c2 = F.o2*K[K_c12];
    const T D_coec_c3 = F.h2*K[K_d6];
    const T D_coec_c4 = F.parthno3*tj[J_hno3];
    const T D_coec_c5 = K[K_c3]*xt56;
    const T D_coec_c6 = K[K_e16]*xt45;
    const T D_coec_c7 = F.hnm*K[K_b24] + tj[J_hno4];
    const T D_coec_c8 = K[K_c9]*xt45 + tj[J_ch2o_hco];
    const T D_coec_c9 = K[K_d35]*xt45 + K[K_d37]*xt44 + tj[J_hocl];
    const T D_coec_c10 = K[K_c1a] + K[K_c1b];
    const T D_coec_c11 = D_coec_c10*xt1 + T(2.4e-10)*F.h2;
    const T D_coec_c12 = T(2)*K[K_a1et];
    const T D_coec_c13 = F.parth2o*(D_coec_c12*xt42 + T(2)*tj[J_h2o]);
    const T D_coec = D_ch3o*D_coec_c1 + D_coec_c0*xt16 + D_coec_c11*xt42 + D_coec_c13*xt2 + D_coec_c2*D_hco + D_coec_c3*xt44 + D_coec_c4*xt4 + D_coec_c5*xt45 + D_coec_c6*xt25 + D_coec_c7*xt21 + D_coec_c8*xt27 + D_coec_c9*xt14 + tj[J_ch3o2h]*xt29 + tj[J_hbr]*xt18 + tj[J_hobr]*xt25;
    const T d_D_coec_1 = D_coec_c1*d_D_ch3o_1 + D_coec_c10*xt42;
    const T d_D_coec_2 = D_coec_c13;
    const T d_D_coec_4 = D_coec_c4;
    const T d_D_coec_14 = D_coec_c9;
    const T d_D_coec_16 = D_coec_c0;
    const T d_D_coec_18 = tj[J_hbr];
    const T d_D_coec_21 = D_coec_c7;
    const T d_D_coec_25 = D_coec_c6 + tj[J_hobr];
    const T d_D_coec_27 = D_coec_c2*d_D_hco_27 + D_coec_c8;
    const T d_D_coec_28 = D_coec_c1*d_D_ch3o_28;
    const T d_D_coec_29 = D_coec_c1*d_D_ch3o_29 + tj[J_ch3o2h];
    const T d_D_coec_42 = D_coec_c1*d_D_ch3o_42 + D_coec_c11 + D_coec_c12*F.parth2o*xt2;
    const T d_D_coec_43 = D_coec_c2*d_D_hco_43;
    const T d_D_coec_44 = D_coec_c2*d_D_hco_44 + D_coec_c3 + K[K_d37]*xt14;
    const T d_D_coec_45 = D_coec_c2*d_D_hco_45 + D_coec_c5 + K[K_c9]*xt27 + K[K_d35]*xt14 + K[K_e16]*xt25;
    const T d_D_coec_49 = D_coec_c1*d_D_ch3o_49;
    const T d_D_coec_50 = D_coec_c2*d_D_hco_50;
    const T d_D_coec_52 = D_coec_c1*d_D_ch3o_52;
    const T d_D_coec_56 = K[K_c3]*xt45;
    const T D_argum_c0 = T(4)*D_coea;
    const T D_argum_c1 = D_argum_c0*D_coec + (D_coeb*D_coeb);
    const T D_argum_c2 = T(2)*D_coeb;
    const T D_argum_c3 = T(4)*D_coec;
    const bool sel_D_argum = (D_argum_c1) >= (T(0));
    const T D_argum = sel_D_argum ? T(D_argum_c1) : T(T(0));
    const T d_D_argum_1 = sel_D_argum ? T(D_argum_c0*d_D_coec_1 + D_argum_c2*d_D_coeb_1) : T(T(0));
    const T d_D_argum_2 = sel_D_argum ? T(D_argum_c0*d_D_coec_2) : T(T(0));
    const T d_D_argum_4 = sel_D_argum ? T(D_argum_c0*d_D_coec_4 + D_argum_c2*d_D_coeb_4) : T(T(0));
    const T d_D_argum_8 = sel_D_argum ? T(D_argum_c2*d_D_coeb_8 + D_argum_c3*d_D_coea_8) : T(T(0));
    const T d_D_argum_12 = sel_D_argum ? T(D_argum_c2*d_D_coeb_12) : T(T(0));
    const T d_D_argum_14 = sel_D_argum ? T(D_argum_c0*d_D_coec_14 + D_argum_c2*d_D_coeb_14) : T(T(0));
    const T d_D_argum_16 = sel_D_argum ? T(D_argum_c0*d_D_coec_16 + D_argum_c2*d_D_coeb_16 + D_argum_c3*d_D_coea_16) : T(T(0));
    const T d_D_argum_18 = sel_D_argum ? T(D_argum_c0*d_D_coec_18 + D_argum_c2*d_D_coeb_18) : T(T(0));
    const T d_D_argum_21 = sel_D_argum ? T(D_argum_c0*d_D_coec_21 + D_argum_c2*d_D_coeb_21) : T(T(0));
    const T d_D_argum_25 = sel_D_argum ? T(D_argum_c0*d_D_coec_25) : T(T(0));
    const T d_D_argum_27 = sel_D_argum ? T(D_argum_c0*d_D_coec_27 + D_argum_c2*d_D_coeb_27 + D_argum_c3*d_D_coea_27) : T(T(0));
    const T d_D_argum_28 = sel_D_argum ? T(D_argum_c0*d_D_coec_28 + D_argum_c2*d_D_coeb_28) : T(T(0));
    const T d_D_argum_29 = sel_D_argum ? T(D_argum_c0*d_D_coec_29 + D_argum_c2*d_D_coeb_29) : T(T(0));
    const T d_D_argum_42 = sel_D_argum ? T(D_argum_c0*d_D_coec_42) : T(T(0));
    const T d_D_argum_43 = sel_D_argum ? T(D_argum_c0*d_D_coec_43 + D_argum_c2*d_D_coeb_43 + D_argum_c3*d_D_coea_43) : T(T(0));
    const T d_D_argum_44 = sel_D_argum ? T(D_argum_c0*d_D_coec_44 + D_argum_c2*d_D_coeb_44 + D_argum_c3*d_D_coea_44) : T(T(0));
    const T d_D_argum_45 = sel_D_argum ? T(D_argum_c0*d_D_coec_45 + D_argum_c2*d_D_coeb_45 + D_argum_c3*d_D_coea_45) : T(T(0));
    const T d_D_argum_46 = sel_D_argum ? T(D_argum_c2*d_D_coeb_46 + D_argum_c3*d_D_coea_46) : T(T(0));
    const T d_D_argum_47 = sel_D_argum ? T(D_argum_c2*d_D_coeb_47 + D_argum_c3*d_D_coea_47) : T(T(0));
    const T d_D_argum_48 = sel_D_argum ? T(D_argum_c2*d_D_coeb_48) : T(T(0));
    const T d_D_argum_49 = sel_D_argum ? T(D_argum_c0*d_D_coec_49 + D_argum_c2*d_D_coeb_49 + D_argum_c3*d_D_coea_49) : T(T(0));
    const T d_D_argum_50 = sel_D_argum ? T(D_argum_c0*d_D_coec_50 + D_argum_c2*d_D_coeb_50 + D_argum_c3*d_D_coea_50) : T(T(0));
    const T d_D_argum_52 = sel_D_argum ? T(D_argum_c0*d_D_coec_52 + D_argum_c2*d_D_coeb_52 + D_argum_c3*d_D_coea_52) : T(T(0));
    const T d_D_argum_53 = sel_D_argum ? T(D_argum_c2*d_D_coeb_53 + D_argum_c3*d_D_coea_53) : T(T(0));
    const T d_D_argum_55 = sel_D_argum ? T(D_argum_c2*d_D_coeb_55 + D_argum_c3*d_D_coea_55) : T(T(0));
    const T d_D_argum_56 = sel_D_argum ? T(D_argum_c0*d_D_coec_56) : T(T(0));
    {  // row 43
    const T rs43 = nt_rscale<T>(nt_exp_hi(x[43]), fh);
        const T dj43_c0 = nt_div<T>(T(1), D_coea);
        const T dj43_c1 = nt_div<T>(dj43_c0, T(2));
        const T dj43_c2 = sqrt(D_argum);
        const T dj43_c3 = nt_div<T>(dj43_c0, T(4)*dj43_c2);
        const T dj43_c4 = nt_div<T>(-D_coeb + dj43_c2, T(2)*(D_coea*D_coea));
        J[321] = (-d_D_argum_1*dj43_c3 + d_D_coeb_1*dj43_c1) * (cs1 * rs43);
        J[331] = (-d_D_argum_2*dj43_c3) * (cs2 * rs43);
        J[319] = (-d_D_argum_4*dj43_c3 + d_D_coeb_4*dj43_c1) * (cs4 * rs43);
        J[322] = (-d_D_argum_8*dj43_c3 + d_D_coea_8*dj43_c4 + d_D_coeb_8*dj43_c1) * (cs8 * rs43);
        J[330] = (-d_D_argum_12*dj43_c3 + d_D_coeb_12*dj43_c1) * (cs12 * rs43);
        J[323] = (-d_D_argum_14*dj43_c3 + d_D_coeb_14*dj43_c1) * (cs14 * rs43);
        J[326] = (-d_D_argum_16*dj43_c3 + d_D_coea_16*dj43_c4 + d_D_coeb_16*dj43_c1) * (cs16 * rs43);
        J[325] = (-d_D_argum_18*dj43_c3 + d_D_coeb_18*dj43_c1) * (cs18 * rs43);
        J[320] = (-d_D_argum_21*dj43_c3 + d_D_coeb_21*dj43_c1) * (cs21 * rs43);
        J[317] = (-d_D_argum_25*dj43_c3) * (cs25 * rs43);
        J[329] = (-d_D_argum_27*dj43_c3 + d_D_coea_27*dj43_c4 + d_D_coeb_27*dj43_c1) * (cs27 * rs43);
        J[328] = (-d_D_argum_28*dj43_c3 + d_D_coeb_28*dj43_c1) * (cs28 * rs43);
        J[316] = (-d_D_argum_29*dj43_c3 + d_D_coeb_29*dj43_c1) * (cs29 * rs43);
        J[318] = (-d_D_argum_42*dj43_c3) * (cs42 * rs43);
        J[337] = (-d_D_argum_43*dj43_c3 + d_D_coea_43*dj43_c4 + d_D_coeb_43*dj43_c1 + T(1)) * (cs43 * rs43);
        J[334] = (-d_D_argum_44*dj43_c3 + d_D_coea_44*dj43_c4 + d_D_coeb_44*dj43_c1) * (cs44 * rs43);
        J[333] = (-d_D_argum_45*dj43_c3 + d_D_coea_45*dj43_c4 + d_D_coeb_45*dj43_c1) * (cs45 * rs43);
        J[339] = (-d_D_argum_46*dj43_c3 + d_D_coea_46*dj43_c4 + d_D_coeb_46*dj43_c1) * (cs46 * rs43);
        J[338] = (-d_D_argum_47*dj43_c3 + d_D_coea_47*dj43_c4 + d_D_coeb_47*dj43_c1) * (cs47 * rs43);
        J[332] = (-d_D_argum_48*dj43_c3 + d_D_coeb_48*dj43_c1) * (cs48 * rs43);
        J[340] = (-d_D_argum_49*dj43_c3 + d_D_coea_49*dj43_c4 + d_D_coeb_49*dj43_c1) * (cs49 * rs43);
        J[336] = (-d_D_argum_50*dj43_c3 + d_D_coea_50*dj43_c4 + d_D_coeb_50*dj43_c1) * (cs50 * rs43);
        J[341] = (-d_D_argum_52*dj43_c3 + d_D_coea_52*dj43_c4 + d_D_coeb_52*dj43_c1) * (cs52 * rs43);
        J[335] = (-d_D_argum_53*dj43_c3 + d_D_coea_53*dj43_c4 + d_D_coeb_53*dj43_c1) * (cs53 * rs43);
        J[327] = (-d_D_argum_55*dj43_c3 + d_D_coea_55*dj43_c4 + d_D_coeb_55*dj43_c1) * (cs55 * rs43);
        J[324] = (-d_D_argum_56*dj43_c3) * (cs56 * rs43);
    }
}

// residual rows [1, 4, 6, 11, 18, 22, 24, 27, 29, 33, 39, 45, 46, 51] (day equations, FP64)
template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>
__device__ __forceinline__ void nt_residual_day_w4_1(const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {
    R[1] = -ck0[1] + x[1]*(F.dt*(K[K_c1a]*x[42] + K[K_c1b]*x[42] + K[K_c1c]*x[42] + K[K_c2]*x[43] + K[K_d5]*x[44]) + T(1));
    R[4] = -F.dt*(K[K_b22]*x[43]*x[48] + het[0]*x[13]*x[2] + het[1]*x[12]*x[13] + T(2)*het[2]*x[2]*x[5] + het[3]*x[12]*x[5] + het[5]*x[19]*x[2]) - ck0[4] + x[4]*(F.dt*(F.parthno3*(K[K_b27]*x[43] + tj[J_hno3]) + F.rain_hno3) + T(1));
    const T dr6_c0 = T(3)*x[42];
    R[6] = F.dt*F.rain_hcl*x[12] - F.dt*(x[30]*(K[K_d90]*dr6_c0 + T(3)*tj[J_cfc11]) + x[31]*(T(2)*K[K_d91]*x[42] + T(2)*tj[J_cfc12]) + x[32]*(K[K_d92]*dr6_c0 + T(3)*tj[J_cfc113]) + x[33]*(T(4)*K[K_d93]*x[42] + T(4)*tj[J_ccl4]) + x[34]*(T(3)*K[K_d94]*x[43] + T(3)*tj[J_ch3ccl3]) + x[35]*(K[K_d95]*x[43] + tj[J_ch3cl]) + x[36]*(K[K_d96]*x[42] + K[K_d97]*x[43] + tj[J_hcfc22]) + x[38]*(K[K_e52]*x[42] + tj[J_h1211])) - ck0[6] + x[6];
    R[11] = -ck0[11] + x[11];
    R[18] = -F.dt*(K[K_c19]*x[27]*x[50] + K[K_e7]*x[47]*x[50]) - ck0[18] + x[18]*(F.dt*(F.parthbr*(K[K_e11]*x[43] + K[K_e9]*x[42] + tj[J_hbr]) + F.rain_hbr + het[7]*x[25] + het[8]*x[14]) + T(1));
    const T dr22_c0 = T(2)*x[52];
    const T dr22_c1 = T(3)*x[42];
    R[22] = F.dt*(x[44]*(F.h2*K[K_d6] + K[K_c10]*x[27] + K[K_d36]*x[48] + K[K_d37]*x[14] + K[K_d5]*x[1] + K[K_d7]*x[47]) + x[52]*(K[K_d31]*x[48] + K[K_d33]*x[47] + K[K_d60]*dr22_c0 + K[K_d62]*dr22_c0 + K[K_d9]*x[43] + K[K_e5a]*x[53] + K[K_e5c]*x[53])) - F.dt*(F.parthcl*x[12]*(K[K_d11]*x[43] + tj[J_hcl]) + tj[J_brcl]*x[26] + T(2)*tj[J_cl2]*x[15] + tj[J_clno2]*x[17] + tj[J_oclo]*x[9] + x[13]*(K[K_d32]*x[45] + tj[J_clono2_cl] + tj[J_clono2_clo]) + x[14]*(K[K_d34]*x[43] + K[K_d35]*x[45] + tj[J_hocl]) + x[24]*(T(2)*F.hnm*K[K_d61] + T(2)*tj[J_cl2o2]) + x[30]*(K[K_d90]*dr22_c1 + T(3)*tj[J_cfc11]) + x[31]*(T(2)*K[K_d91]*x[42] + T(2)*tj[J_cfc12]) + x[32]*(K[K_d92]*dr22_c1 + T(3)*tj[J_cfc113]) + x[33]*(T(4)*K[K_d93]*x[42] + T(4)*tj[J_ccl4]) + x[34]*(T(3)*K[K_d94]*x[43] + T(3)*tj[J_ch3ccl3]) + x[35]*(K[K_d95]*x[43] + tj[J_ch3cl]) + x[36]*(K[K_d96]*x[42] + K[K_d97]*x[43] + tj[J_hcfc22])) - ck0[22] + x[22];
    R[24] = -F.dt*K[K_d60]*(x[52]*x[52]) - ck0[24] + x[24]*(F.dt*(F.hnm*K[K_d61] + tj[J_cl2o2]) + T(1));
    R[29] = -F.dt*K[K_c7]*x[28]*x[47] - ck0[29] + x[29]*(F.dt*(K[K_c17a]*x[43] + K[K_c17b]*x[43] + tj[J_ch3o2h]) + T(1));
    R[33] = -ck0[33] + x[33]*(F.dt*(K[K_d93]*x[42] + tj[J_ccl4]) + T(1));
    R[39] = -ck0[39] + x[39]*(F.dt*(K[K_e53]*x[42] + tj[J_h1301]) + T(1));
    const T D_ch3o = nt_div<T>(K[K_c1b]*x[1]*x[42] + tj[J_ch3o2h]*x[29] + x[28]*(T(2)*K[K_c14]*x[28] + K[K_c18]*x[52] + K[K_c5]*x[49]), F.o2*K[K_c15]);
    R[27] = -F.dt*(D_ch3o*F.o2*K[K_c15] + K[K_c17b]*x[29]*x[43] + K[K_c1c]*x[1]*x[42] + K[K_c3]*x[45]*x[56]) - ck0[27] + x[27]*(F.dt*(K[K_c10]*x[44] + K[K_c19]*x[50] + K[K_c8]*x[43] + K[K_c9]*x[45] + tj[J_ch2o_co] + tj[J_ch2o_hco]) + T(1));
    const T D_r1 = nt_div<T>(K[K_a2]*x[55] + K[K_a6]*x[43] + K[K_a6b]*x[47] + K[K_b4]*x[49] + K[K_d2]*x[44] + tj[J_o3_o1d] + tj[J_o3_o3p], F.o2*K[K_hk2]);
    R[45] = -D_r1*x[46] + x[45];
    R[46] = x[46] + nt_div<T>(-x[7], D_r1 + T(1));
    const T D_r7 = nt_div<T>(tj[J_no], F.o2*K[K_b7] + K[K_b6]*x[49]);
    R[51] = -D_r7*x[49] + x[51];
}

// scaled Jacobian rows [1, 3, 8, 9, 15, 17, 18, 20, 22, 31, 34, 36, 39, 45, 46, 47, 55] (day equations) into their stored A slots
template <typename T, typename FF, typename PK, typename PJ>
__device__ __forceinline__ void nt_jacobian_day_w4_1(const FF& F, PK K, PK tj, PK het, const double* __restrict__ x, double floor_, PJ J) {
    const int fh = nt_exp_hi(floor_);
    const T xt0 = nt_cvt<T>(x[0]);
    const T xt1 = nt_cvt<T>(x[1]);
    const T xt2 = nt_cvt<T>(x[2]);
    const T xt3 = nt_cvt<T>(x[3]);
    const T xt4 = nt_cvt<T>(x[4]);
    const T xt5 = nt_cvt<T>(x[5]);
    const T xt6 = nt_cvt<T>(x[6]);
    const T xt7 = nt_cvt<T>(x[7]);
    const T xt8 = nt_cvt<T>(x[8]);
    const T xt9 = nt_cvt<T>(x[9]);
    const T xt10 = nt_cvt<T>(x[10]);
    const T xt11 = nt_cvt<T>(x[11]);
    const T xt12 = nt_cvt<T>(x[12]);
    const T xt13 = nt_cvt<T>(x[13]);
    const T xt14 = nt_cvt<T>(x[14]);
    const T xt15 = nt_cvt<T>(x[15]);
    const T xt16 = nt_cvt<T>(x[16]);
    const T xt17 = nt_cvt<T>(x[17]);
    const T xt18 = nt_cvt<T>(x[18]);
    const T xt19 = nt_cvt<T>(x[19]);
    const T xt20 = nt_cvt<T>(x[20]);
    const T xt21 = nt_cvt<T>(x[21]);
    const T xt22 = nt_cvt<T>(x[22]);
    const T xt23 = nt_cvt<T>(x[23]);
    const T xt24 = nt_cvt<T>(x[24]);
    const T xt25 = nt_cvt<T>(x[25]);
    const T xt26 = nt_cvt<T>(x[26]);
    const T xt27 = nt_cvt<T>(x[27]);
    const T xt28 = nt_cvt<T>(x[28]);
    const T xt29 = nt_cvt<T>(x[29]);
    const T xt30 = nt_cvt<T>(x[30]);
    const T xt31 = nt_cvt<T>(x[31]);
    const T xt32 = nt_cvt<T>(x[32]);
    const T xt33 = nt_cvt<T>(x[33]);
    const T xt34 = nt_cvt<T>(x[34]);
    const T xt35 = nt_cvt<T>(x[35]);
    const T xt36 = nt_cvt<T>(x[36]);
    const T xt37 = nt_cvt<T>(x[37]);
    const T xt38 = nt_cvt<T>(x[38]);
    const T xt39 = nt_cvt<T>(x[39]);
    const T xt40 = nt_cvt<T>(x[40]);
    const T xt41 = nt_cvt<T>(x[41]);
    const T xt42 = nt_cvt<T>(x[42]);
    const T xt43 = nt_cvt<T>(x[43]);
    const T xt44 = nt_cvt<T>(x[44]);
    const T xt45 = nt_cvt<T>(x[45]);
    const T xt46 = nt_cvt<T>(x[46]);
    const T xt47 = nt_cvt<T>(x[47]);
    const T xt48 = nt_cvt<T>(x[48]);
    const T xt49 = nt_cvt<T>(x[49]);
    const T xt50 = nt_cvt<T>(x[50]);
    const T xt51 = nt_cvt<T>(x[51]);
    const T xt52 = nt_cvt<T>(x[52]);
    const T xt53 = nt_cvt<T>(x[53]);
    const T xt54 = nt_cvt<T>(x[54]);
    const T xt55 = nt_cvt<T>(x[55]);
    const T xt56 = nt_cvt<T>(x[56]);
    const T cs0 = nt_scale<T>(nt_exp_hi(x[0]), fh);
    const T cs1 = nt_scale<T>(nt_exp_hi(x[1]), fh);
    const T cs4 = nt_scale<T>(nt_exp_hi(x[4]), fh);
    const T cs5 = nt_scale<T>(nt_exp_hi(x[5]), fh);
    const T cs7 = nt_scale<T>(nt_exp_hi(x[7]), fh);
    const T cs8 = nt_scale<T>(nt_exp_hi(x[8]), fh);
    const T cs9 = nt_scale<T>(nt_exp_hi(x[9]), fh);
    const T cs12 = nt_scale<T>(nt_exp_hi(x[12]), fh);
    const T cs13 = nt_scale<T>(nt_exp_hi(x[13]), fh);
    const T cs14 = nt_scale<T>(nt_exp_hi(x[14]), fh);
    const T cs15 = nt_scale<T>(nt_exp_hi(x[15]), fh);
    const T cs16 = nt_scale<T>(nt_exp_hi(x[16]), fh);
    const T cs17 = nt_scale<T>(nt_exp_hi(x[17]), fh);
    const T cs18 = nt_scale<T>(nt_exp_hi(x[18]), fh);
    const T cs19 = nt_scale<T>(nt_exp_hi(x[19]), fh);
    const T cs21 = nt_scale<T>(nt_exp_hi(x[21]), fh);
    const T cs24 = nt_scale<T>(nt_exp_hi(x[24]), fh);
    const T cs25 = nt_scale<T>(nt_exp_hi(x[25]), fh);
    const T cs26 = nt_scale<T>(nt_exp_hi(x[26]), fh);
    const T cs27 = nt_scale<T>(nt_exp_hi(x[27]), fh);
    const T cs30 = nt_scale<T>(nt_exp_hi(x[30]), fh);
    const T cs31 = nt_scale<T>(nt_exp_hi(x[31]), fh);
    const T cs32 = nt_scale<T>(nt_exp_hi(x[32]), fh);
    const T cs33 = nt_scale<T>(nt_exp_hi(x[33]), fh);
    const T cs34 = nt_scale<T>(nt_exp_hi(x[34]), fh);
    const T cs35 = nt_scale<T>(nt_exp_hi(x[35]), fh);
    const T cs36 = nt_scale<T>(nt_exp_hi(x[36]), fh);
    const T cs39 = nt_scale<T>(nt_exp_hi(x[39]), fh);
    const T cs42 = nt_scale<T>(nt_exp_hi(x[42]), fh);
    const T cs43 = nt_scale<T>(nt_exp_hi(x[43]), fh);
    const T cs44 = nt_scale<T>(nt_exp_hi(x[44]), fh);
    const T cs45 = nt_scale<T>(nt_exp_hi(x[45]), fh);
    const T cs46 = nt_scale<T>(nt_exp_hi(x[46]), fh);
    const T cs47 = nt_scale<T>(nt_exp_hi(x[47]), fh);
    const T cs48 = nt_scale<T>(nt_exp_hi(x[48]), fh);
    const T cs49 = nt_scale<T>(nt_exp_hi(x[49]), fh);
    const T cs50 = nt_scale<T>(nt_exp_hi(x[50]), fh);
    const T cs51 = nt_scale<T>(nt_exp_hi(x[51]), fh);
    const T cs52 = nt_scale<T>(nt_exp_hi(x[52]), fh);
    const T cs53 = nt_scale<T>(nt_exp_hi(x[53]), fh);
    const T cs54 = nt_scale<T>(nt_exp_hi(x[54]), fh);
    const T cs55 = nt_scale<T>(nt_exp_hi(x[55]), fh);
    {  // row 1
    const T rs1 = nt_rscale<T>(nt_exp_hi(x[1]), fh);
        const T dj1_c0 = F.dt*xt1;
        J[157] = (F.dt*(K[K_c1a]*xt42 + K[K_c1b]*xt42 + K[K_c1c]*xt42 + K[K_c2]*xt43 + K[K_d5]*xt44) + T(1)) * (cs1 * rs1);
        J[156] = (dj1_c0*(K[K_c1a] + K[K_c1b] + K[K_c1c])) * (cs42 * rs1);
        J[159] = (K[K_c2]*dj1_c0) * (cs43 * rs1);
        J[158] = (K[K_d5]*dj1_c0) * (cs44 * rs1);
    }
    {  // row 3
    const T rs3 = nt_rscale<T>(nt_exp_hi(x[3]), fh);
        const T dj3_c0 = T(2)*F.dt;
        const T dj3_c1 = K[K_b39]*dj3_c0;
        const T dj3_c2 = K[K_b6]*dj3_c0;
        J[20] = (-dj3_c1*xt42) * (cs0 * rs3);
        J[23] = (F.dt*F.rain_hno3) * (cs4 * rs3);
        J[22] = (-dj3_c1*xt0) * (cs42 * rs3);
        J[24] = (dj3_c2*xt51) * (cs49 * rs3);
        J[21] = (dj3_c2*xt49) * (cs51 * rs3);
    }
    {  // row 9
    const T rs9 = nt_rscale<T>(nt_exp_hi(x[9]), fh);
        const T dj9_c0 = F.dt*K[K_e5a];
        J[100] = (F.dt*tj[J_oclo] + T(1)) * (cs9 * rs9);
        J[102] = (-dj9_c0*xt53) * (cs52 * rs9);
        J[101] = (-dj9_c0*xt52) * (cs53 * rs9);
    }
    {  // row 15
    const T rs15 = nt_rscale<T>(nt_exp_hi(x[15]), fh);
        J[63] = (-F.dt*(het[1]*xt13 + het[4]*xt14)) * (cs12 * rs15);
        J[61] = (-F.dt*het[1]*xt12) * (cs13 * rs15);
        J[62] = (-F.dt*(K[K_d37]*xt44 + het[4]*xt12)) * (cs14 * rs15);
        J[60] = (F.dt*tj[J_cl2] + T(1)) * (cs15 * rs15);
        J[64] = (-F.dt*K[K_d37]*xt14) * (cs44 * rs15);
        J[65] = (-T(2)*F.dt*K[K_d62]*xt52) * (cs52 * rs15);
    }
    {  // row 17
    const T rs17 = nt_rscale<T>(nt_exp_hi(x[17]), fh);
        const T dj17_c0 = F.dt*het[3];
        const T dj17_c1 = F.dt*K[K_d36];
        J[26] = (-dj17_c0*xt12) * (cs5 * rs17);
        J[27] = (-dj17_c0*xt5) * (cs12 * rs17);
        J[25] = (F.dt*tj[J_clno2] + T(1)) * (cs17 * rs17);
        J[29] = (-dj17_c1*xt48) * (cs44 * rs17);
        J[28] = (-dj17_c1*xt44) * (cs48 * rs17);
    }
    {  // row 18
    const T rs18 = nt_rscale<T>(nt_exp_hi(x[18]), fh);
        const T dj18_c0 = F.dt*xt18;
        const T dj18_c1 = F.dt*xt50;
        const T dj18_c2 = F.parthbr*dj18_c0;
        J[183] = (dj18_c0*het[8]) * (cs14 * rs18);
        J[184] = (F.dt*(F.parthbr*(K[K_e11]*xt43 + K[K_e9]*xt42 + tj[J_hbr]) + F.rain_hbr + het[7]*xt25 + het[8]*xt14) + T(1)) * (cs18 * rs18);
        J[181] = (dj18_c0*het[7]) * (cs25 * rs18);
        J[185] = (-K[K_c19]*dj18_c1) * (cs27 * rs18);
        J[182] = (K[K_e9]*dj18_c2) * (cs42 * rs18);
        J[187] = (K[K_e11]*dj18_c2) * (cs43 * rs18);
        J[188] = (-K[K_e7]*dj18_c1) * (cs47 * rs18);
        J[186] = (-F.dt*(K[K_c19]*xt27 + K[K_e7]*xt47)) * (cs50 * rs18);
    }
    {  // row 20
    const T rs20 = nt_rscale<T>(nt_exp_hi(x[20]), fh);
        const T dj20_c0 = T(2)*F.dt;
        const T dj20_c1 = K[K_b39]*dj20_c0;
        const T dj20_c2 = F.parthno3*K[K_b27];
        const T dj20_c3 = F.dt*xt48;
        const T dj20_c4 = T(2)*K[K_b12];
        const T dj20_c5 = K[K_b6]*dj20_c0;
        J[233] = (-dj20_c1*xt42) * (cs0 * rs20);
        J[237] = (-F.dt*(F.parthno3*tj[J_hno3] + dj20_c2*xt43)) * (cs4 * rs20);
        J[232] = (-F.dt*(T(2)*F.hnm*K[K_b32] + T(2)*tj[J_n2o5])) * (cs5 * rs20);
        J[235] = (-F.dt*(K[K_d32]*xt45 + tj[J_clono2_cl] + tj[J_clono2_clo])) * (cs13 * rs20);
        J[229] = (-F.dt*tj[J_clno2]) * (cs17 * rs20);
        J[230] = (-F.dt*(K[K_e8]*xt45 + tj[J_brono2])) * (cs19 * rs20);
        J[238] = (-F.dt*(F.hnm*K[K_b24] + K[K_b28]*xt43 + tj[J_hno4])) * (cs21 * rs20);
        J[236] = (-dj20_c1*xt0) * (cs42 * rs20);
        J[243] = (-F.dt*(K[K_b28]*xt21 + dj20_c2*xt4) + K[K_b22]*dj20_c3) * (cs43 * rs20);
        J[241] = (K[K_d36]*dj20_c3) * (cs44 * rs20);
        J[240] = (-F.dt*(K[K_d32]*xt13 + K[K_e8]*xt19)) * (cs45 * rs20);
        J[244] = (K[K_b23]*dj20_c3) * (cs47 * rs20);
        J[239] = (F.dt*(K[K_b22]*xt43 + K[K_b23]*xt47 + K[K_d31]*xt52 + K[K_d36]*xt44 + K[K_e13]*xt53 + dj20_c4*xt54)) * (cs48 * rs20);
        J[245] = (dj20_c5*xt51) * (cs49 * rs20);
        J[234] = (dj20_c5*xt49) * (cs51 * rs20);
        J[246] = (K[K_d31]*dj20_c3) * (cs52 * rs20);
        J[242] = (K[K_e13]*dj20_c3) * (cs53 * rs20);
        J[231] = (dj20_c3*dj20_c4) * (cs54 * rs20);
    }
    {  // row 22
    const T rs22 = nt_rscale<T>(nt_exp_hi(x[22]), fh);
        const T dj22_c0 = F.dt*xt44;
        const T dj22_c1 = T(3)*xt42;
        const T dj22_c2 = T(2)*K[K_d91];
        const T dj22_c3 = T(4)*K[K_d93];
        const T dj22_c4 = T(3)*K[K_d94];
        const T dj22_c5 = F.dt*xt52;
        const T dj22_c6 = T(2)*K[K_d60];
        const T dj22_c7 = T(2)*K[K_d62];
        J[141] = (K[K_d5]*dj22_c0) * (cs1 * rs22);
        J[140] = (-F.dt*tj[J_oclo]) * (cs9 * rs22);
        J[144] = (-F.dt*F.parthcl*(K[K_d11]*xt43 + tj[J_hcl])) * (cs12 * rs22);
        J[135] = (-F.dt*(K[K_d32]*xt45 + tj[J_clono2_cl] + tj[J_clono2_clo])) * (cs13 * rs22);
        J[142] = (-F.dt*(K[K_d34]*xt43 + K[K_d35]*xt45 + tj[J_hocl]) + K[K_d37]*dj22_c0) * (cs14 * rs22);
        J[133] = (-T(2)*F.dt*tj[J_cl2]) * (cs15 * rs22);
        J[128] = (-F.dt*tj[J_clno2]) * (cs17 * rs22);
        J[138] = (-F.dt*(T(2)*F.hnm*K[K_d61] + T(2)*tj[J_cl2o2])) * (cs24 * rs22);
        J[132] = (-F.dt*tj[J_brcl]) * (cs26 * rs22);
        J[143] = (K[K_c10]*dj22_c0) * (cs27 * rs22);
        J[137] = (-F.dt*(K[K_d90]*dj22_c1 + T(3)*tj[J_cfc11])) * (cs30 * rs22);
        J[131] = (-F.dt*(dj22_c2*xt42 + T(2)*tj[J_cfc12])) * (cs31 * rs22);
        J[127] = (-F.dt*(K[K_d92]*dj22_c1 + T(3)*tj[J_cfc113])) * (cs32 * rs22);
        J[129] = (-F.dt*(dj22_c3*xt42 + T(4)*tj[J_ccl4])) * (cs33 * rs22);
        J[136] = (-F.dt*(dj22_c4*xt43 + T(3)*tj[J_ch3ccl3])) * (cs34 * rs22);
        J[134] = (-F.dt*(K[K_d95]*xt43 + tj[J_ch3cl])) * (cs35 * rs22);
        J[130] = (-F.dt*(K[K_d96]*xt42 + K[K_d97]*xt43 + tj[J_hcfc22])) * (cs36 * rs22);
        J[139] = (-F.dt*(T(3)*K[K_d90]*xt30 + T(3)*K[K_d92]*xt32 + K[K_d96]*xt36 + dj22_c2*xt31 + dj22_c3*xt33)) * (cs42 * rs22);
        J[149] = (-F.dt*(F.parthcl*K[K_d11]*xt12 + K[K_d34]*xt14 + K[K_d95]*xt35 + K[K_d97]*xt36 + dj22_c4*xt34) + K[K_d9]*dj22_c5) * (cs43 * rs22);
        J[147] = (F.dt*(F.h2*K[K_d6] + K[K_c10]*xt27 + K[K_d36]*xt48 + K[K_d37]*xt14 + K[K_d5]*xt1 + K[K_d7]*xt47)) * (cs44 * rs22);
        J[146] = (-F.dt*(K[K_d32]*xt13 + K[K_d35]*xt14)) * (cs45 * rs22);
        J[150] = (F.dt*(K[K_d33]*xt52 + K[K_d7]*xt44)) * (cs47 * rs22);
        J[145] = (F.dt*(K[K_d31]*xt52 + K[K_d36]*xt44)) * (cs48 * rs22);
        J[151] = (F.dt*(K[K_d31]*xt48 + K[K_d33]*xt47 + K[K_d9]*xt43 + K[K_e5a]*xt53 + K[K_e5c]*xt53 + dj22_c6*xt52 + dj22_c7*xt52 + xt52*(dj22_c6 + dj22_c7))) * (cs52 * rs22);
        J[148] = (dj22_c5*(K[K_e5a] + K[K_e5c])) * (cs53 * rs22);
    }
    {  // row 31
    const T rs31 = nt_rscale<T>(nt_exp_hi(x[31]), fh);
        J[41] = (F.dt*(K[K_d91]*xt42 + tj[J_cfc12]) + T(1)) * (cs31 * rs31);
        J[42] = (F.dt*K[K_d91]*xt31) * (cs42 * rs31);
    }
    {  // row 34
    const T rs34 = nt_rscale<T>(nt_exp_hi(x[34]), fh);
        J[93] = (F.dt*(K[K_d94]*xt43 + tj[J_ch3ccl3]) + T(1)) * (cs34 * rs34);
        J[94] = (F.dt*K[K_d94]*xt34) * (cs43 * rs34);
    }
    {  // row 36
    const T rs36 = nt_rscale<T>(nt_exp_hi(x[36]), fh);
        const T dj36_c0 = F.dt*xt36;
        J[38] = (F.dt*(K[K_d96]*xt42 + K[K_d97]*xt43 + tj[J_hcfc22]) + T(1)) * (cs36 * rs36);
        J[39] = (K[K_d96]*dj36_c0) * (cs42 * rs36);
        J[40] = (K[K_d97]*dj36_c0) * (cs43 * rs36);
    }
    {  // row 39
    const T rs39 = nt_rscale<T>(nt_exp_hi(x[39]), fh);
        J[50] = (F.dt*(K[K_e53]*xt42 + tj[J_h1301]) + T(1)) * (cs39 * rs39);
        J[51] = (F.dt*K[K_e53]*xt39) * (cs42 * rs39);
    }
    const T D_hco_c0 = nt_div<T>(T(1), F.o2*K[K_c12]);
    const T D_hco_c1 = D_hco_c0*(K[K_c10]*xt44 + K[K_c19]*xt50 + K[K_c8]*xt43 + K[K_c9]*xt45 + tj[J_ch2o_hco]);
    const T D_hco_c2 = D_hco_c0*xt27;
    const T D_hco = D_hco_c1*xt27;
    const T d_D_hco_27 = D_hco_c1;
    const T d_D_hco_43 = D_hco_c2*K[K_c8];
    const T d_D_hco_44 = D_hco_c2*K[K_c10];
    const T d_D_hco_45 = D_hco_c2*K[K_c9];
    const T d_D_hco_50 = D_hco_c2*K[K_c19];
    {  // row 8
    const T rs8 = nt_rscale<T>(nt_exp_hi(x[8]), fh);
        const T dj8_c0 = F.dt*F.o2*K[K_c12];
        J[160] = (F.dt*K[K_a36]*xt43 + T(1)) * (cs8 * rs8);
        J[161] = (-F.dt*tj[J_ch2o_co] - d_D_hco_27*dj8_c0) * (cs27 * rs8);
        J[165] = (F.dt*K[K_a36]*xt8 - d_D_hco_43*dj8_c0) * (cs43 * rs8);
        J[163] = (-d_D_hco_44*dj8_c0) * (cs44 * rs8);
        J[162] = (-d_D_hco_45*dj8_c0) * (cs45 * rs8);
        J[164] = (-d_D_hco_50*dj8_c0) * (cs50 * rs8);
    }
    const T D_r1_c0 = nt_div<T>(T(1), F.o2*K[K_hk2]);
    const T D_r1 = D_r1_c0*(K[K_a2]*xt55 + K[K_a6]*xt43 + K[K_a6b]*xt47 + K[K_b4]*xt49 + K[K_d2]*xt44 + tj[J_o3_o1d] + tj[J_o3_o3p]);
    const T d_D_r1_43 = D_r1_c0*K[K_a6];
    const T d_D_r1_44 = D_r1_c0*K[K_d2];
    const T d_D_r1_47 = D_r1_c0*K[K_a6b];
    const T d_D_r1_49 = D_r1_c0*K[K_b4];
    const T d_D_r1_55 = D_r1_c0*K[K_a2];
    {  // row 45
    const T rs45 = nt_rscale<T>(nt_exp_hi(x[45]), fh);
        J[280] = (-d_D_r1_43*xt46) * (cs43 * rs45);
        J[279] = (-d_D_r1_44*xt46) * (cs44 * rs45);
        J[282] = (-D_r1) * (cs46 * rs45);
        J[281] = (-d_D_r1_47*xt46) * (cs47 * rs45);
        J[283] = (-d_D_r1_49*xt46) * (cs49 * rs45);
        J[278] = (-d_D_r1_55*xt46) * (cs55 * rs45);
    }
    {  // row 46
    const T rs46 = nt_rscale<T>(nt_exp_hi(x[46]), fh);
        const T dj46_c0 = D_r1 + T(1);
        const T dj46_c1 = nt_div<T>(xt7, (dj46_c0*dj46_c0));
        J[355] = (nt_div<T>(T(-1), dj46_c0)) * (cs7 * rs46);
        J[358] = (d_D_r1_43*dj46_c1) * (cs43 * rs46);
        J[357] = (d_D_r1_44*dj46_c1) * (cs44 * rs46);
        J[359] = (d_D_r1_47*dj46_c1) * (cs47 * rs46);
        J[360] = (d_D_r1_49*dj46_c1) * (cs49 * rs46);
        J[356] = (d_D_r1_55*dj46_c1) * (cs55 * rs46);
    }
    const T D_r4_c0 = F.h2*K[K_a19] + K[K_a36]*xt8 + K[K_a5]*xt45;
    const T D_r4_c1 = F.o2*K[K_a1] + K[K_a2]*xt46 + T(8.049999999999999e-11)*xt47;
    const T D_r4_c2 = nt_div<T>(T(1), D_r4_c1);
    const T D_r4_c3 = nt_div<T>(D_r4_c0, (D_r4_c1*D_r4_c1));
    const T D_r4 = D_r4_c0*D_r4_c2;
    const T d_D_r4_8 = D_r4_c2*K[K_a36];
    const T d_D_r4_45 = D_r4_c2*K[K_a5];
    const T d_D_r4_46 = -D_r4_c3*K[K_a2];
    const T d_D_r4_47 = -T(8.049999999999999e-11)*D_r4_c3;
    {  // row 55
    const T rs55 = nt_rscale<T>(nt_exp_hi(x[55]), fh);
        J[205] = (-d_D_r4_8*xt43) * (cs8 * rs55);
        J[207] = (-D_r4) * (cs43 * rs55);
        J[206] = (-d_D_r4_45*xt43) * (cs45 * rs55);
        J[209] = (-d_D_r4_46*xt43) * (cs46 * rs55);
        J[208] = (-d_D_r4_47*xt43) * (cs47 * rs55);
    }
    const T D_r6_c0 = F.o2*K[K_a1];
    const T D_r6_c1 = D_r4*D_r6_c0 + K[K_a30]*xt16 + K[K_a6]*xt46 + K[K_c8]*xt27 + K[K_d8]*xt52 + K[K_e10]*xt53;
    const T D_r6_c2 = T(2)*K[K_a27];
    const T D_r6_c3 = D_r6_c2*xt47 + K[K_a17]*xt43 + K[K_a26]*xt49 + K[K_a6b]*xt46 + K[K_a7]*xt45 + K[K_d10]*xt44 + K[K_d33]*xt52 + K[K_d7]*xt44 + K[K_e15]*xt53 + K[K_e7]*xt50 + T(8.049999999999999e-11)*xt55;
    const T D_r6_c4 = nt_div<T>(T(1), D_r6_c3);
    const T D_r6_c5 = D_r6_c0*D_r6_c4;
    const T D_r6_c6 = nt_div<T>(D_r6_c1, (D_r6_c3*D_r6_c3));
    const T D_r6 = D_r6_c1*D_r6_c4;
    const T d_D_r6_8 = D_r6_c5*d_D_r4_8;
    const T d_D_r6_16 = D_r6_c4*K[K_a30];
    const T d_D_r6_27 = D_r6_c4*K[K_c8];
    const T d_D_r6_43 = -D_r6_c6*K[K_a17];
    const T d_D_r6_44 = D_r6_c6*(-K[K_d10] - K[K_d7]);
    const T d_D_r6_45 = D_r6_c5*d_D_r4_45 - D_r6_c6*K[K_a7];
    const T d_D_r6_46 = D_r6_c4*K[K_a6] + D_r6_c5*d_D_r4_46 - D_r6_c6*K[K_a6b];
    const T d_D_r6_47 = -D_r6_c2*D_r6_c6 + D_r6_c5*d_D_r4_47;
    const T d_D_r6_49 = -D_r6_c6*K[K_a26];
    const T d_D_r6_50 = -D_r6_c6*K[K_e7];
    const T d_D_r6_52 = D_r6_c4*K[K_d8] - D_r6_c6*K[K_d33];
    const T d_D_r6_53 = D_r6_c4*K[K_e10] - D_r6_c6*K[K_e15];
    const T d_D_r6_55 = -T(8.049999999999999e-11)*D_r6_c6;
    {  // row 47
    const T rs47 = nt_rscale<T>(nt_exp_hi(x[47]), fh);
        J[342] = (-d_D_r6_8*xt43) * (cs8 * rs47);
        J[343] = (-d_D_r6_16*xt43) * (cs16 * rs47);
        J[345] = (-d_D_r6_27*xt43) * (cs27 * rs47);
        J[350] = (-D_r6 - d_D_r6_43*xt43) * (cs43 * rs47);
        J[347] = (-d_D_r6_44*xt43) * (cs44 * rs47);
        J[346] = (-d_D_r6_45*xt43) * (cs45 * rs47);
        J[352] = (-d_D_r6_46*xt43) * (cs46 * rs47);
        J[351] = (-d_D_r6_47*xt43 + T(1)) * (cs47 * rs47);
        J[353] = (-d_D_r6_49*xt43) * (cs49 * rs47);
        J[349] = (-d_D_r6_50*xt43) * (cs50 * rs47);
        J[354] = (-d_D_r6_52*xt43) * (cs52 * rs47);
        J[348] = (-d_D_r6_53*xt43) * (cs53 * rs47);
        J[344] = (-d_D_r6_55*xt43) * (cs55 * rs47);
    }
}

// residual rows [2, 7, 17, 19, 25, 26, 31, 35, 36, 40, 42, 47, 48, 49, 54] (day equations, FP64)
template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>
__device__ __forceinline__ void nt_residual_day_w4_2(const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {
    const T dr2_c0 = x[29]*x[43];
    R[2] = -F.dt*(F.h2*K[K_a19]*x[43] + F.parthcl*K[K_d11]*x[12]*x[43] + F.parthno3*K[K_b27]*x[43]*x[4] + K[K_a30]*x[16]*x[43] + K[K_a31]*(x[43]*x[43]) + K[K_c17a]*dr2_c0 + K[K_c17b]*dr2_c0 + K[K_c2]*x[1]*x[43] + K[K_c8]*x[27]*x[43] + x[47]*(K[K_a17]*x[43] + T(1.6e-12)*x[55])) - ck0[2] + x[2]*(F.dt*F.parth2o*(K[K_a1et]*x[42] + tj[J_h2o]) + T(1));
    R[17] = -F.dt*(K[K_d36]*x[44]*x[48] + het[3]*x[12]*x[5]) - ck0[17] + x[17]*(F.dt*tj[J_clno2] + T(1));
    R[19] = -F.dt*K[K_e13]*x[48]*x[53] - ck0[19] + x[19]*(F.dt*(K[K_e8]*x[45] + het[5]*x[2] + tj[J_brono2]) + T(1));
    R[25] = -F.dt*(K[K_e15]*x[47]*x[53] + het[5]*x[19]*x[2]) - ck0[25] + x[25]*(F.dt*(K[K_e16]*x[45] + het[6]*x[12] + het[7]*x[18] + tj[J_hobr]) + T(1));
    R[26] = -F.dt*(K[K_e5c]*x[52]*x[53] + het[6]*x[12]*x[25] + het[8]*x[14]*x[18]) - ck0[26] + x[26]*(F.dt*tj[J_brcl] + T(1));
    R[31] = -ck0[31] + x[31]*(F.dt*(K[K_d91]*x[42] + tj[J_cfc12]) + T(1));
    R[35] = -ck0[35] + x[35]*(F.dt*(K[K_d95]*x[43] + tj[J_ch3cl]) + T(1));
    R[36] = -ck0[36] + x[36]*(F.dt*(K[K_d96]*x[42] + K[K_d97]*x[43] + tj[J_hcfc22]) + T(1));
    R[40] = F.dt*F.rain_hbr*x[18] - F.dt*(x[37]*(K[K_e50]*x[42] + K[K_e51]*x[43] + tj[J_ch3br]) + x[38]*(K[K_e52]*x[42] + tj[J_h1211]) + x[39]*(K[K_e53]*x[42] + tj[J_h1301]) + x[41]*(T(2)*K[K_e54]*x[43] + T(2)*tj[J_ch2br2])) - ck0[40] + x[40];
    R[42] = nt_div<T>(-tj[J_o3_o1d]*x[46], F.n2*K[K_hk4] + F.o2*K[K_hk5]) + x[42];
    const T D_r4 = nt_div<T>(F.h2*K[K_a19] + K[K_a36]*x[8] + K[K_a5]*x[45], F.o2*K[K_a1] + K[K_a2]*x[46] + T(8.049999999999999e-11)*x[47]);
    const T D_r7 = nt_div<T>(tj[J_no], F.o2*K[K_b7] + K[K_b6]*x[49]);
    const T D_r8 = nt_div<T>(K[K_b9]*x[46], K[K_b12]*x[48] + tj[J_no3_no2] + tj[J_no3_no]);
    R[54] = -D_r8*x[48] + x[54];
    const T D_r5 = nt_div<T>(D_r8*tj[J_no3_no] + K[K_b3]*x[45] + tj[J_no2], K[K_a26]*x[47] + K[K_b4]*x[46] + K[K_c5]*x[28] + K[K_d4]*x[52] + K[K_e4]*x[53]);
    R[48] = nt_div<T>(-x[20], D_r5*D_r7 + D_r5 + D_r8 + T(1)) + x[48];
    R[49] = -D_r5*x[48] + x[49];
    const T D_r6 = nt_div<T>(D_r4*F.o2*K[K_a1] + K[K_a30]*x[16] + K[K_a6]*x[46] + K[K_c8]*x[27] + K[K_d8]*x[52] + K[K_e10]*x[53], K[K_a17]*x[43] + K[K_a26]*x[49] + T(2)*K[K_a27]*x[47] + K[K_a6b]*x[46] + K[K_a7]*x[45] + K[K_d10]*x[44] + K[K_d33]*x[52] + K[K_d7]*x[44] + K[K_e15]*x[53] + K[K_e7]*x[50] + T(8.049999999999999e-11)*x[55]);
    R[47] = -D_r6*x[43] + x[47];
    const T D_t06_c0 = tj[J_hocl]*x[14];
    const T D_t06_c1 = K[K_d33]*x[47]*x[52];
    const bool sel_D_t06 = (D_t06_c0) <= (D_t06_c1);
    const T D_t06 = sel_D_t06 ? T(D_t06_c0) : T(D_t06_c1);
    const T D_t07_c0 = K[K_e5c]*x[52]*x[53];
    const T D_t07_c1 = tj[J_brcl]*x[26];
    const bool sel_D_t07 = (D_t07_c0) <= (D_t07_c1);
    const T D_t07 = sel_D_t07 ? T(D_t07_c0) : T(D_t07_c1);
    const T D_t09_c0 = K[K_e15]*x[47]*x[53];
    const T D_t09_c1 = tj[J_hobr]*x[25];
    const bool sel_D_t09 = (D_t09_c0) <= (D_t09_c1);
    const T D_t09 = sel_D_t09 ? T(D_t09_c0) : T(D_t09_c1);
    const T dr7_c0 = T(2)*x[45];
    const T dr7_c1 = nt_div<T>(T(2)*tj[J_no3_no], fmax(T(1e-30), tj[J_no3_no2] + tj[J_no3_no]));
    R[7] = -F.dt*(T(2)*F.o2*tj[J_o2] + K[K_a26]*x[47]*x[49] + K[K_c5]*x[28]*x[49]) + F.dt*(D_t06 + T(2)*D_t07 + D_t09 + K[K_b3]*dr7_c0*x[48] + K[K_b9]*dr7_c1*x[46]*x[48] + K[K_d3]*dr7_c0*x[52] + nt_div<T>(T(2)*K[K_d60]*tj[J_cl2o2]*(x[52]*x[52]), F.hnm*K[K_d61] + tj[J_cl2o2]) + T(2)*K[K_e5b]*x[52]*x[53] + T(2)*K[K_e6]*(x[53]*x[53]) + T(2)*K[K_hk1]*(x[45]*x[45]) + K[K_hk3]*dr7_c0*x[46] + dr7_c1*tj[J_clono2_cl]*x[13] + x[45]*(K[K_a5]*x[43] + K[K_a7]*x[47]) + x[46]*(K[K_a2]*x[55] + K[K_a6]*x[43] + K[K_a6b]*x[47])) - ck0[7] + x[7];
}

// scaled Jacobian rows [0, 4, 5, 6, 12, 13, 16, 25, 27, 29, 30, 33, 38, 40, 42, 50, 52, 53] (day equations) into their stored A slots
template <typename T, typename FF, typename PK, typename PJ>
__device__ __forceinline__ void nt_jacobian_day_w4_2(const FF& F, PK K, PK tj, PK het, const double* __restrict__ x, double floor_, PJ J) {
    const int fh = nt_exp_hi(floor_);
    const T xt0 = nt_cvt<T>(x[0]);
    const T xt1 = nt_cvt<T>(x[1]);
    const T xt2 = nt_cvt<T>(x[2]);
    const T xt3 = nt_cvt<T>(x[3]);
    const T xt4 = nt_cvt<T>(x[4]);
    const T xt5 = nt_cvt<T>(x[5]);
    const T xt6 = nt_cvt<T>(x[6]);
    const T xt7 = nt_cvt<T>(x[7]);
    const T xt8 = nt_cvt<T>(x[8]);
    const T xt9 = nt_cvt<T>(x[9]);
    const T xt10 = nt_cvt<T>(x[10]);
    const T xt11 = nt_cvt<T>(x[11]);
    const T xt12 = nt_cvt<T>(x[12]);
    const T xt13 = nt_cvt<T>(x[13]);
    const T xt14 = nt_cvt<T>(x[14]);
    const T xt15 = nt_cvt<T>(x[15]);
    const T xt16 = nt_cvt<T>(x[16]);
    const T xt17 = nt_cvt<T>(x[17]);
    const T xt18 = nt_cvt<T>(x[18]);
    const T xt19 = nt_cvt<T>(x[19]);
    const T xt20 = nt_cvt<T>(x[20]);
    const T xt21 = nt_cvt<T>(x[21]);
    const T xt22 = nt_cvt<T>(x[22]);
    const T xt23 = nt_cvt<T>(x[23]);
    const T xt24 = nt_cvt<T>(x[24]);
    const T xt25 = nt_cvt<T>(x[25]);
    const T xt26 = nt_cvt<T>(x[26]);
    const T xt27 = nt_cvt<T>(x[27]);
    const T xt28 = nt_cvt<T>(x[28]);
    const T xt29 = nt_cvt<T>(x[29]);
    const T xt30 = nt_cvt<T>(x[30]);
    const T xt31 = nt_cvt<T>(x[31]);
    const T xt32 = nt_cvt<T>(x[32]);
    const T xt33 = nt_cvt<T>(x[33]);
    const T xt34 = nt_cvt<T>(x[34]);
    const T xt35 = nt_cvt<T>(x[35]);
    const T xt36 = nt_cvt<T>(x[36]);
    const T xt37 = nt_cvt<T>(x[37]);
    const T xt38 = nt_cvt<T>(x[38]);
    const T xt39 = nt_cvt<T>(x[39]);
    const T xt40 = nt_cvt<T>(x[40]);
    const T xt41 = nt_cvt<T>(x[41]);
    const T xt42 = nt_cvt<T>(x[42]);
    const T xt43 = nt_cvt<T>(x[43]);
    const T xt44 = nt_cvt<T>(x[44]);
    const T xt45 = nt_cvt<T>(x[45]);
    const T xt46 = nt_cvt<T>(x[46]);
    const T xt47 = nt_cvt<T>(x[47]);
    const T xt48 = nt_cvt<T>(x[48]);
    const T xt49 = nt_cvt<T>(x[49]);
    const T xt50 = nt_cvt<T>(x[50]);
    const T xt51 = nt_cvt<T>(x[51]);
    const T xt52 = nt_cvt<T>(x[52]);
    const T xt53 = nt_cvt<T>(x[53]);
    const T xt54 = nt_cvt<T>(x[54]);
    const T xt55 = nt_cvt<T>(x[55]);
    const T xt56 = nt_cvt<T>(x[56]);
    const T cs0 = nt_scale<T>(nt_exp_hi(x[0]), fh);
    const T cs1 = nt_scale<T>(nt_exp_hi(x[1]), fh);
    const T cs2 = nt_scale<T>(nt_exp_hi(x[2]), fh);
    const T cs4 = nt_scale<T>(nt_exp_hi(x[4]), fh);
    const T cs5 = nt_scale<T>(nt_exp_hi(x[5]), fh);
    const T cs12 = nt_scale<T>(nt_exp_hi(x[12]), fh);
    const T cs13 = nt_scale<T>(nt_exp_hi(x[13]), fh);
    const T cs14 = nt_scale<T>(nt_exp_hi(x[14]), fh);
    const T cs16 = nt_scale<T>(nt_exp_hi(x[16]), fh);
    const T cs18 = nt_scale<T>(nt_exp_hi(x[18]), fh);
    const T cs19 = nt_scale<T>(nt_exp_hi(x[19]), fh);
    const T cs22 = nt_scale<T>(nt_exp_hi(x[22]), fh);
    const T cs23 = nt_scale<T>(nt_exp_hi(x[23]), fh);
    const T cs25 = nt_scale<T>(nt_exp_hi(x[25]), fh);
    const T cs27 = nt_scale<T>(nt_exp_hi(x[27]), fh);
    const T cs28 = nt_scale<T>(nt_exp_hi(x[28]), fh);
    const T cs29 = nt_scale<T>(nt_exp_hi(x[29]), fh);
    const T cs30 = nt_scale<T>(nt_exp_hi(x[30]), fh);
    const T cs31 = nt_scale<T>(nt_exp_hi(x[31]), fh);
    const T cs32 = nt_scale<T>(nt_exp_hi(x[32]), fh);
    const T cs33 = nt_scale<T>(nt_exp_hi(x[33]), fh);
    const T cs34 = nt_scale<T>(nt_exp_hi(x[34]), fh);
    const T cs35 = nt_scale<T>(nt_exp_hi(x[35]), fh);
    const T cs36 = nt_scale<T>(nt_exp_hi(x[36]), fh);
    const T cs37 = nt_scale<T>(nt_exp_hi(x[37]), fh);
    const T cs38 = nt_scale<T>(nt_exp_hi(x[38]), fh);
    const T cs39 = nt_scale<T>(nt_exp_hi(x[39]), fh);
    const T cs41 = nt_scale<T>(nt_exp_hi(x[41]), fh);
    const T cs42 = nt_scale<T>(nt_exp_hi(x[42]), fh);
    const T cs43 = nt_scale<T>(nt_exp_hi(x[43]), fh);
    const T cs44 = nt_scale<T>(nt_exp_hi(x[44]), fh);
    const T cs45 = nt_scale<T>(nt_exp_hi(x[45]), fh);
    const T cs46 = nt_scale<T>(nt_exp_hi(x[46]), fh);
    const T cs47 = nt_scale<T>(nt_exp_hi(x[47]), fh);
    const T cs48 = nt_scale<T>(nt_exp_hi(x[48]), fh);
    const T cs49 = nt_scale<T>(nt_exp_hi(x[49]), fh);
    const T cs50 = nt_scale<T>(nt_exp_hi(x[50]), fh);
    const T cs52 = nt_scale<T>(nt_exp_hi(x[52]), fh);
    const T cs53 = nt_scale<T>(nt_exp_hi(x[53]), fh);
    const T cs54 = nt_scale<T>(nt_exp_hi(x[54]), fh);
    const T cs56 = nt_scale<T>(nt_exp_hi(x[56]), fh);
    {  // row 0
    const T rs0 = nt_rscale<T>(nt_exp_hi(x[0]), fh);
        const T dj0_c0 = K[K_b38] + K[K_b39];
        J[76] = (F.dt*(dj0_c0*xt42 + tj[J_n2o]) + T(1)) * (cs0 * rs0);
        J[77] = (F.dt*dj0_c0*xt0) * (cs42 * rs0);
    }
    {  // row 4
    const T rs4 = nt_rscale<T>(nt_exp_hi(x[4]), fh);
        const T dj4_c0 = T(2)*het[2];
        const T dj4_c1 = F.dt*K[K_b22];
        J[122] = (-F.dt*(dj4_c0*xt5 + het[0]*xt13 + het[5]*xt19)) * (cs2 * rs4);
        J[120] = (F.dt*(F.parthno3*(K[K_b27]*xt43 + tj[J_hno3]) + F.rain_hno3) + T(1)) * (cs4 * rs4);
        J[118] = (-F.dt*(dj4_c0*xt2 + het[3]*xt12)) * (cs5 * rs4);
        J[121] = (-F.dt*(het[1]*xt13 + het[3]*xt5)) * (cs12 * rs4);
        J[119] = (-F.dt*(het[0]*xt2 + het[1]*xt12)) * (cs13 * rs4);
        J[117] = (-F.dt*het[5]*xt2) * (cs19 * rs4);
        J[124] = (F.dt*F.parthno3*K[K_b27]*xt4 - dj4_c1*xt48) * (cs43 * rs4);
        J[123] = (-dj4_c1*xt43) * (cs48 * rs4);
    }
    {  // row 5
    const T rs5 = nt_rscale<T>(nt_exp_hi(x[5]), fh);
        const T dj5_c0 = F.dt*xt5;
        const T dj5_c1 = F.dt*K[K_b12];
        J[74] = (dj5_c0*het[2]) * (cs2 * rs5);
        J[72] = (F.dt*(F.hnm*K[K_b32] + het[2]*xt2 + het[3]*xt12 + tj[J_n2o5]) + T(1)) * (cs5 * rs5);
        J[73] = (dj5_c0*het[3]) * (cs12 * rs5);
        J[75] = (-dj5_c1*xt54) * (cs48 * rs5);
        J[71] = (-dj5_c1*xt48) * (cs54 * rs5);
    }
    {  // row 6
    const T rs6 = nt_rscale<T>(nt_exp_hi(x[6]), fh);
        const T dj6_c0 = T(3)*xt42;
        const T dj6_c1 = T(2)*K[K_d91];
        const T dj6_c2 = T(4)*K[K_d93];
        const T dj6_c3 = T(3)*K[K_d94];
        J[9] = (F.dt*F.rain_hcl) * (cs12 * rs6);
        J[7] = (-F.dt*(K[K_d90]*dj6_c0 + T(3)*tj[J_cfc11])) * (cs30 * rs6);
        J[4] = (-F.dt*(dj6_c1*xt42 + T(2)*tj[J_cfc12])) * (cs31 * rs6);
        J[0] = (-F.dt*(K[K_d92]*dj6_c0 + T(3)*tj[J_cfc113])) * (cs32 * rs6);
        J[2] = (-F.dt*(dj6_c2*xt42 + T(4)*tj[J_ccl4])) * (cs33 * rs6);
        J[6] = (-F.dt*(dj6_c3*xt43 + T(3)*tj[J_ch3ccl3])) * (cs34 * rs6);
        J[5] = (-F.dt*(K[K_d95]*xt43 + tj[J_ch3cl])) * (cs35 * rs6);
        J[3] = (-F.dt*(K[K_d96]*xt42 + K[K_d97]*xt43 + tj[J_hcfc22])) * (cs36 * rs6);
        J[1] = (-F.dt*(K[K_e52]*xt42 + tj[J_h1211])) * (cs38 * rs6);
        J[8] = (-F.dt*(T(3)*K[K_d90]*xt30 + T(3)*K[K_d92]*xt32 + K[K_d96]*xt36 + K[K_e52]*xt38 + dj6_c1*xt31 + dj6_c2*xt33)) * (cs42 * rs6);
        J[10] = (-F.dt*(K[K_d95]*xt35 + K[K_d97]*xt36 + dj6_c3*xt34)) * (cs43 * rs6);
    }
    {  // row 12
    const T rs12 = nt_rscale<T>(nt_exp_hi(x[12]), fh);
        const T dj12_c0 = F.dt*xt44;
        const T dj12_c1 = F.dt*xt12;
        const T dj12_c2 = F.dt*K[K_d9];
        J[250] = (-K[K_d5]*dj12_c0) * (cs1 * rs12);
        J[247] = (dj12_c1*het[3]) * (cs5 * rs12);
        J[253] = (F.dt*(F.parthcl*(K[K_d11]*xt43 + tj[J_hcl]) + F.rain_hcl + het[1]*xt13 + het[3]*xt5 + het[4]*xt14 + het[6]*xt25) + T(1)) * (cs12 * rs12);
        J[249] = (dj12_c1*het[1]) * (cs13 * rs12);
        J[251] = (dj12_c1*het[4]) * (cs14 * rs12);
        J[248] = (dj12_c1*het[6]) * (cs25 * rs12);
        J[252] = (-K[K_c10]*dj12_c0) * (cs27 * rs12);
        J[255] = (F.parthcl*K[K_d11]*dj12_c1 - dj12_c2*xt52) * (cs43 * rs12);
        J[254] = (-F.dt*(F.h2*K[K_d6] + K[K_c10]*xt27 + K[K_d5]*xt1 + K[K_d7]*xt47)) * (cs44 * rs12);
        J[256] = (-K[K_d7]*dj12_c0) * (cs47 * rs12);
        J[257] = (-dj12_c2*xt43) * (cs52 * rs12);
    }
    {  // row 13
    const T rs13 = nt_rscale<T>(nt_exp_hi(x[13]), fh);
        const T dj13_c0 = F.dt*xt13;
        const T dj13_c1 = F.dt*K[K_d31];
        J[89] = (dj13_c0*het[0]) * (cs2 * rs13);
        J[88] = (dj13_c0*het[1]) * (cs12 * rs13);
        J[87] = (F.dt*(K[K_d32]*xt45 + het[0]*xt2 + het[1]*xt12 + tj[J_clono2_cl] + tj[J_clono2_clo]) + T(1)) * (cs13 * rs13);
        J[91] = (K[K_d32]*dj13_c0) * (cs45 * rs13);
        J[90] = (-dj13_c1*xt52) * (cs48 * rs13);
        J[92] = (-dj13_c1*xt48) * (cs52 * rs13);
    }
    {  // row 16
    const T rs16 = nt_rscale<T>(nt_exp_hi(x[16]), fh);
        J[189] = (F.dt*(F.rain_h2o2 + K[K_a30]*xt43 + tj[J_h2o2]) + T(1)) * (cs16 * rs16);
        J[190] = (F.dt*K[K_a30]*xt16) * (cs43 * rs16);
        J[191] = (-T(2)*F.dt*K[K_a27]*xt47) * (cs47 * rs16);
    }
    {  // row 25
    const T rs25 = nt_rscale<T>(nt_exp_hi(x[25]), fh);
        const T dj25_c0 = F.dt*het[5];
        const T dj25_c1 = F.dt*xt25;
        const T dj25_c2 = F.dt*K[K_e15];
        J[83] = (-dj25_c0*xt19) * (cs2 * rs25);
        J[82] = (dj25_c1*het[6]) * (cs12 * rs25);
        J[81] = (dj25_c1*het[7]) * (cs18 * rs25);
        J[79] = (-dj25_c0*xt2) * (cs19 * rs25);
        J[80] = (F.dt*(K[K_e16]*xt45 + het[6]*xt12 + het[7]*xt18 + tj[J_hobr]) + T(1)) * (cs25 * rs25);
        J[84] = (K[K_e16]*dj25_c1) * (cs45 * rs25);
        J[86] = (-dj25_c2*xt53) * (cs47 * rs25);
        J[85] = (-dj25_c2*xt47) * (cs53 * rs25);
    }
    {  // row 29
    const T rs29 = nt_rscale<T>(nt_exp_hi(x[29]), fh);
        const T dj29_c0 = F.dt*K[K_c7];
        J[35] = (-dj29_c0*xt47) * (cs28 * rs29);
        J[34] = (F.dt*(K[K_c17a]*xt43 + K[K_c17b]*xt43 + tj[J_ch3o2h]) + T(1)) * (cs29 * rs29);
        J[36] = (F.dt*xt29*(K[K_c17a] + K[K_c17b])) * (cs43 * rs29);
        J[37] = (-dj29_c0*xt28) * (cs47 * rs29);
    }
    {  // row 30
    const T rs30 = nt_rscale<T>(nt_exp_hi(x[30]), fh);
        J[95] = (F.dt*(K[K_d90]*xt42 + tj[J_cfc11]) + T(1)) * (cs30 * rs30);
        J[96] = (F.dt*K[K_d90]*xt30) * (cs42 * rs30);
    }
    {  // row 33
    const T rs33 = nt_rscale<T>(nt_exp_hi(x[33]), fh);
        J[32] = (F.dt*(K[K_d93]*xt42 + tj[J_ccl4]) + T(1)) * (cs33 * rs33);
        J[33] = (F.dt*K[K_d93]*xt33) * (cs42 * rs33);
    }
    {  // row 38
    const T rs38 = nt_rscale<T>(nt_exp_hi(x[38]), fh);
        J[30] = (F.dt*(K[K_e52]*xt42 + tj[J_h1211]) + T(1)) * (cs38 * rs38);
        J[31] = (F.dt*K[K_e52]*xt38) * (cs42 * rs38);
    }
    {  // row 40
    const T rs40 = nt_rscale<T>(nt_exp_hi(x[40]), fh);
        const T dj40_c0 = T(2)*K[K_e54];
        J[16] = (F.dt*F.rain_hbr) * (cs18 * rs40);
        J[13] = (-F.dt*(K[K_e50]*xt42 + K[K_e51]*xt43 + tj[J_ch3br])) * (cs37 * rs40);
        J[11] = (-F.dt*(K[K_e52]*xt42 + tj[J_h1211])) * (cs38 * rs40);
        J[12] = (-F.dt*(K[K_e53]*xt42 + tj[J_h1301])) * (cs39 * rs40);
        J[15] = (-F.dt*(dj40_c0*xt43 + T(2)*tj[J_ch2br2])) * (cs41 * rs40);
        J[14] = (-F.dt*(K[K_e50]*xt37 + K[K_e52]*xt38 + K[K_e53]*xt39)) * (cs42 * rs40);
        J[17] = (-F.dt*(K[K_e51]*xt37 + dj40_c0*xt41)) * (cs43 * rs40);
    }
    {  // row 42
    const T rs42 = nt_rscale<T>(nt_exp_hi(x[42]), fh);
        J[99] = (nt_div<T>(-tj[J_o3_o1d], F.n2*K[K_hk4] + F.o2*K[K_hk5])) * (cs46 * rs42);
    }
    const T D_ch3o_c0 = K[K_c1b]*xt42;
    const T D_ch3o_c1 = K[K_c14]*xt28;
    const T D_ch3o_c2 = K[K_c18]*xt52 + K[K_c5]*xt49;
    const T D_ch3o_c3 = nt_div<T>(T(1), F.o2*K[K_c15]);
    const T D_ch3o_c4 = D_ch3o_c3*xt28;
    const T D_ch3o = D_ch3o_c3*(D_ch3o_c0*xt1 + tj[J_ch3o2h]*xt29 + xt28*(T(2)*D_ch3o_c1 + D_ch3o_c2));
    const T d_D_ch3o_1 = D_ch3o_c0*D_ch3o_c3;
    const T d_D_ch3o_28 = D_ch3o_c3*(T(4)*D_ch3o_c1 + D_ch3o_c2);
    const T d_D_ch3o_29 = D_ch3o_c3*tj[J_ch3o2h];
    const T d_D_ch3o_42 = D_ch3o_c3*K[K_c1b]*xt1;
    const T d_D_ch3o_49 = D_ch3o_c4*K[K_c5];
    const T d_D_ch3o_52 = D_ch3o_c4*K[K_c18];
    {  // row 27
    const T rs27 = nt_rscale<T>(nt_exp_hi(x[27]), fh);
        const T dj27_c0 = F.dt*K[K_c1c];
        const T dj27_c1 = F.dt*F.o2*K[K_c15];
        const T dj27_c2 = F.dt*K[K_c17b];
        const T dj27_c3 = F.dt*xt27;
        const T dj27_c4 = F.dt*K[K_c3];
        J[219] = (-d_D_ch3o_1*dj27_c1 - dj27_c0*xt42) * (cs1 * rs27);
        J[222] = (F.dt*(K[K_c10]*xt44 + K[K_c19]*xt50 + K[K_c8]*xt43 + K[K_c9]*xt45 + tj[J_ch2o_co] + tj[J_ch2o_hco]) + T(1)) * (cs27 * rs27);
        J[221] = (-d_D_ch3o_28*dj27_c1) * (cs28 * rs27);
        J[217] = (-d_D_ch3o_29*dj27_c1 - dj27_c2*xt43) * (cs29 * rs27);
        J[218] = (-d_D_ch3o_42*dj27_c1 - dj27_c0*xt1) * (cs42 * rs27);
        J[226] = (F.dt*K[K_c8]*xt27 - dj27_c2*xt29) * (cs43 * rs27);
        J[224] = (K[K_c10]*dj27_c3) * (cs44 * rs27);
        J[223] = (F.dt*K[K_c9]*xt27 - dj27_c4*xt56) * (cs45 * rs27);
        J[227] = (-d_D_ch3o_49*dj27_c1) * (cs49 * rs27);
        J[225] = (K[K_c19]*dj27_c3) * (cs50 * rs27);
        J[228] = (-d_D_ch3o_52*dj27_c1) * (cs52 * rs27);
        J[220] = (-dj27_c4*xt45) * (cs56 * rs27);
    }
    const T D_r13_c0 = K[K_d32]*xt45 + het[0]*xt2 + het[1]*xt12 + tj[J_clono2_cl] + tj[J_clono2_clo];
    const T D_r13_c1 = nt_div<T>(K[K_d31], D_r13_c0);
    const T D_r13_c2 = nt_div<T>(K[K_d31]*xt48, (D_r13_c0*D_r13_c0));
    const T D_r13 = D_r13_c1*xt48;
    const T d_D_r13_2 = -D_r13_c2*het[0];
    const T d_D_r13_12 = -D_r13_c2*het[1];
    const T d_D_r13_45 = -D_r13_c2*K[K_d32];
    const T d_D_r13_48 = D_r13_c1;
    const T D_r9_c0 = D_r13*het[0];
    const T D_r9_c1 = D_r9_c0*xt2 + K[K_d33]*xt47;
    const T D_r9_c2 = K[K_d35]*xt45 + het[4]*xt12 + tj[J_hocl];
    const T D_r9_c3 = nt_div<T>(T(1), D_r9_c2);
    const T D_r9_c4 = D_r9_c3*het[0]*xt2;
    const T D_r9_c5 = nt_div<T>(D_r9_c1, (D_r9_c2*D_r9_c2));
    const T D_r9 = D_r9_c1*D_r9_c3;
    const T d_D_r9_2 = D_r9_c0*D_r9_c3 + D_r9_c4*d_D_r13_2;
    const T d_D_r9_12 = D_r9_c4*d_D_r13_12 - D_r9_c5*het[4];
    const T d_D_r9_45 = D_r9_c3*d_D_r13_45*het[0]*xt2 - D_r9_c5*K[K_d35];
    const T d_D_r9_47 = D_r9_c3*K[K_d33];
    const T d_D_r9_48 = D_r9_c4*d_D_r13_48;
    const T D_r10_c0 = nt_div<T>(K[K_d60], F.hnm*K[K_d61] + tj[J_cl2o2]);
    const T D_r10 = D_r10_c0*xt52;
    const T d_D_r10_52 = D_r10_c0;
    const T D_r12_c0 = nt_div<T>(K[K_e5c], tj[J_brcl]);
    const T D_r12 = D_r12_c0*xt53;
    const T d_D_r12_53 = D_r12_c0;
    const T D_r11_c0 = K[K_d10]*xt47 + K[K_d2]*xt46 + K[K_d37]*xt14 + K[K_d5]*xt1 + K[K_d7]*xt47;
    const T D_r11_c1 = nt_div<T>(T(1), D_r11_c0);
    const T D_r11_c2 = T(2)*tj[J_cl2o2];
    const T D_r11_c3 = D_r10*D_r11_c2 + D_r12*tj[J_brcl] + D_r13*tj[J_clono2_cl] + D_r9*tj[J_hocl] + K[K_c18]*xt28 + K[K_d3]*xt45 + K[K_d4]*xt49 + K[K_d8]*xt43 + K[K_e5b]*xt53;
    const T D_r11_c4 = nt_div<T>(D_r11_c3, (D_r11_c0*D_r11_c0));
    const T D_r11_c5 = D_r11_c1*tj[J_clono2_cl];
    const T D_r11_c6 = D_r11_c1*tj[J_hocl];
    const T D_r11 = D_r11_c1*D_r11_c3;
    const T d_D_r11_1 = -D_r11_c4*K[K_d5];
    const T d_D_r11_2 = D_r11_c5*d_D_r13_2 + D_r11_c6*d_D_r9_2;
    const T d_D_r11_12 = D_r11_c5*d_D_r13_12 + D_r11_c6*d_D_r9_12;
    const T d_D_r11_14 = -D_r11_c4*K[K_d37];
    const T d_D_r11_28 = D_r11_c1*K[K_c18];
    const T d_D_r11_43 = D_r11_c1*K[K_d8];
    const T d_D_r11_45 = D_r11_c1*K[K_d3] + D_r11_c5*d_D_r13_45 + D_r11_c6*d_D_r9_45;
    const T d_D_r11_46 = -D_r11_c4*K[K_d2];
    const T d_D_r11_47 = D_r11_c4*(-K[K_d10] - K[K_d7]) + D_r11_c6*d_D_r9_47;
    const T d_D_r11_48 = D_r11_c5*d_D_r13_48 + D_r11_c6*d_D_r9_48;
    const T d_D_r11_49 = D_r11_c1*K[K_d4];
    const T d_D_r11_52 = D_r11_c1*D_r11_c2*d_D_r10_52;
    const T d_D_r11_53 = D_r11_c1*K[K_e5b] + D_r11_c1*d_D_r12_53*tj[J_brcl];
    {  // row 52
    const T rs52 = nt_rscale<T>(nt_exp_hi(x[52]), fh);
        const T dj52_c0 = D_r11 + T(1);
        const T dj52_c1 = nt_div<T>(xt22, (dj52_c0*dj52_c0));
        J[369] = (d_D_r11_1*dj52_c1) * (cs1 * rs52);
        J[373] = (d_D_r11_2*dj52_c1) * (cs2 * rs52);
        J[372] = (d_D_r11_12*dj52_c1) * (cs12 * rs52);
        J[370] = (d_D_r11_14*dj52_c1) * (cs14 * rs52);
        J[368] = (nt_div<T>(T(-1), dj52_c0)) * (cs22 * rs52);
        J[371] = (d_D_r11_28*dj52_c1) * (cs28 * rs52);
        J[377] = (d_D_r11_43*dj52_c1) * (cs43 * rs52);
        J[375] = (d_D_r11_45*dj52_c1) * (cs45 * rs52);
        J[379] = (d_D_r11_46*dj52_c1) * (cs46 * rs52);
        J[378] = (d_D_r11_47*dj52_c1) * (cs47 * rs52);
        J[374] = (d_D_r11_48*dj52_c1) * (cs48 * rs52);
        J[380] = (d_D_r11_49*dj52_c1) * (cs49 * rs52);
        J[381] = (d_D_r11_52*dj52_c1 + T(1)) * (cs52 * rs52);
        J[376] = (d_D_r11_53*dj52_c1) * (cs53 * rs52);
    }
    const T D_r27_c0 = K[K_e8]*xt45 + tj[J_brono2];
    const T D_r27_c1 = nt_div<T>(K[K_e13], D_r27_c0);
    const T D_r27 = D_r27_c1*xt48;
    const T d_D_r27_45 = nt_div<T>(-K[K_e13]*K[K_e8]*xt48, (D_r27_c0*D_r27_c0));
    const T d_D_r27_48 = D_r27_c1;
    const T D_r28_c0 = K[K_e16]*xt45 + tj[J_hobr];
    const T D_r28_c1 = nt_div<T>(K[K_e15], D_r28_c0);
    const T D_r28 = D_r28_c1*xt47;
    const T d_D_r28_45 = nt_div<T>(-K[K_e15]*K[K_e16]*xt47, (D_r28_c0*D_r28_c0));
    const T d_D_r28_47 = D_r28_c1;
    const T D_r29_c0 = nt_div<T>(K[K_e5c], tj[J_brcl]);
    const T D_r29 = D_r29_c0*xt52;
    const T d_D_r29_52 = D_r29_c0;
    const T D_r30_c0 = K[K_c19]*xt27 + K[K_e2]*xt46 + K[K_e7]*xt47;
    const T D_r30_c1 = nt_div<T>(T(1), D_r30_c0);
    const T D_r30_c2 = T(0.85)*tj[J_brono2];
    const T D_r30_c3 = T(2)*K[K_e6];
    const T D_r30_c4 = D_r27*D_r30_c2 + D_r28*tj[J_hobr] + D_r29*tj[J_brcl] + D_r30_c3*xt53 + K[K_e10]*xt43 + K[K_e3]*xt45 + K[K_e4]*xt49 + K[K_e5a]*xt52 + K[K_e5b]*xt52 + tj[J_bro];
    const T D_r30_c5 = nt_div<T>(D_r30_c4, (D_r30_c0*D_r30_c0));
    const T D_r30_c6 = D_r30_c1*D_r30_c2;
    const T D_r30 = D_r30_c1*D_r30_c4;
    const T d_D_r30_27 = -D_r30_c5*K[K_c19];
    const T d_D_r30_43 = D_r30_c1*K[K_e10];
    const T d_D_r30_45 = D_r30_c1*K[K_e3] + D_r30_c1*d_D_r28_45*tj[J_hobr] + D_r30_c6*d_D_r27_45;
    const T d_D_r30_46 = -D_r30_c5*K[K_e2];
    const T d_D_r30_47 = D_r30_c1*d_D_r28_47*tj[J_hobr] - D_r30_c5*K[K_e7];
    const T d_D_r30_48 = D_r30_c6*d_D_r27_48;
    const T d_D_r30_49 = D_r30_c1*K[K_e4];
    const T d_D_r30_52 = D_r30_c1*d_D_r29_52*tj[J_brcl] + D_r30_c1*(K[K_e5a] + K[K_e5b]);
    const T d_D_r30_53 = D_r30_c1*D_r30_c3;
    {  // row 50
    const T rs50 = nt_rscale<T>(nt_exp_hi(x[50]), fh);
        J[307] = (-d_D_r30_27*xt53) * (cs27 * rs50);
        J[311] = (-d_D_r30_43*xt53) * (cs43 * rs50);
        J[309] = (-d_D_r30_45*xt53) * (cs45 * rs50);
        J[313] = (-d_D_r30_46*xt53) * (cs46 * rs50);
        J[312] = (-d_D_r30_47*xt53) * (cs47 * rs50);
        J[308] = (-d_D_r30_48*xt53) * (cs48 * rs50);
        J[314] = (-d_D_r30_49*xt53) * (cs49 * rs50);
        J[315] = (-d_D_r30_52*xt53) * (cs52 * rs50);
        J[310] = (-D_r30 - d_D_r30_53*xt53) * (cs53 * rs50);
    }
    {  // row 53
    const T rs53 = nt_rscale<T>(nt_exp_hi(x[53]), fh);
        const T dj53_c0 = D_r30 + T(1);
        const T dj53_c1 = nt_div<T>(xt23, (dj53_c0*dj53_c0));
        J[297] = (nt_div<T>(T(-1), dj53_c0)) * (cs23 * rs53);
        J[298] = (d_D_r30_27*dj53_c1) * (cs27 * rs53);
        J[302] = (d_D_r30_43*dj53_c1) * (cs43 * rs53);
        J[300] = (d_D_r30_45*dj53_c1) * (cs45 * rs53);
        J[304] = (d_D_r30_46*dj53_c1) * (cs46 * rs53);
        J[303] = (d_D_r30_47*dj53_c1) * (cs47 * rs53);
        J[299] = (d_D_r30_48*dj53_c1) * (cs48 * rs53);
        J[305] = (d_D_r30_49*dj53_c1) * (cs49 * rs53);
        J[306] = (d_D_r30_52*dj53_c1) * (cs52 * rs53);
        J[301] = (d_D_r30_53*dj53_c1 + T(1)) * (cs53 * rs53);
    }
}

// residual rows [0, 3, 8, 9, 10, 13, 16, 20, 23, 28, 32, 38, 44, 50, 52, 53] (day equations, FP64)
template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>
__device__ __forceinline__ void nt_residual_day_w4_3(const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {
    R[0] = -ck0[0] + x[0]*(F.dt*(tj[J_n2o] + x[42]*(K[K_b38] + K[K_b39])) + T(1));
    R[3] = -T(2)*F.dt*K[K_b39]*x[0]*x[42] + F.dt*(F.rain_hno3*x[4] + T(2)*K[K_b6]*x[49]*x[51]) - ck0[3] + x[3];
    R[9] = -F.dt*K[K_e5a]*x[52]*x[53] - ck0[9] + x[9]*(F.dt*tj[J_oclo] + T(1));
    R[10] = -ck0[10] + x[10];
    R[13] = -F.dt*K[K_d31]*x[48]*x[52] - ck0[13] + x[13]*(F.dt*(K[K_d32]*x[45] + het[0]*x[2] + het[1]*x[12] + tj[J_clono2_cl] + tj[J_clono2_clo]) + T(1));
    R[16] = -F.dt*K[K_a27]*(x[47]*x[47]) - ck0[16] + x[16]*(F.dt*(F.rain_h2o2 + K[K_a30]*x[43] + tj[J_h2o2]) + T(1));
    const T dr20_c0 = F.parthno3*x[4];
    R[20] = F.dt*(T(2)*K[K_b6]*x[49]*x[51] + x[48]*(T(2)*K[K_b12]*x[54] + K[K_b22]*x[43] + K[K_b23]*x[47] + K[K_d31]*x[52] + K[K_d36]*x[44] + K[K_e13]*x[53])) - F.dt*(K[K_b27]*dr20_c0*x[43] + T(2)*K[K_b39]*x[0]*x[42] + K[K_d32]*x[13]*x[45] + K[K_e8]*x[19]*x[45] + dr20_c0*tj[J_hno3] + tj[J_brono2]*x[19] + tj[J_clno2]*x[17] + x[13]*(tj[J_clono2_cl] + tj[J_clono2_clo]) + x[21]*(F.hnm*K[K_b24] + K[K_b28]*x[43] + tj[J_hno4]) + x[5]*(T(2)*F.hnm*K[K_b32] + T(2)*tj[J_n2o5])) - ck0[20] + x[20];
    R[23] = F.dt*(K[K_c19]*x[27]*x[50] + K[K_e7]*x[47]*x[50] + x[53]*(K[K_e13]*x[48] + K[K_e15]*x[47] + K[K_e5c]*x[52])) - F.dt*(F.parthbr*x[18]*(K[K_e11]*x[43] + K[K_e9]*x[42] + tj[J_hbr]) + K[K_e16]*x[25]*x[45] + K[K_e8]*x[19]*x[45] + T(2)*het[7]*x[18]*x[25] + tj[J_brcl]*x[26] + tj[J_brono2]*x[19] + tj[J_hobr]*x[25]) - ck0[23] + x[23];
    R[28] = -F.dt*(F.o2*K[K_c4]*x[56] + K[K_c17a]*x[29]*x[43]) - ck0[28] + x[28]*(F.dt*(T(2)*K[K_c14]*x[28] + K[K_c18]*x[52] + K[K_c5]*x[49] + K[K_c7]*x[47]) + T(1));
    R[32] = -ck0[32] + x[32]*(F.dt*(K[K_d92]*x[42] + tj[J_cfc113]) + T(1));
    R[38] = -ck0[38] + x[38]*(F.dt*(K[K_e52]*x[42] + tj[J_h1211]) + T(1));
    const T D_hco = nt_div<T>(x[27]*(K[K_c10]*x[44] + K[K_c19]*x[50] + K[K_c8]*x[43] + K[K_c9]*x[45] + tj[J_ch2o_hco]), F.o2*K[K_c12]);
    R[8] = -F.dt*(D_hco*F.o2*K[K_c12] + F.co2*tj[J_co2] + tj[J_ch2o_co]*x[27]) - ck0[8] + x[8]*(F.dt*K[K_a36]*x[43] + T(1));
    const T D_r13 = nt_div<T>(K[K_d31]*x[48], K[K_d32]*x[45] + het[0]*x[2] + het[1]*x[12] + tj[J_clono2_cl] + tj[J_clono2_clo]);
    const T D_r9 = nt_div<T>(D_r13*het[0]*x[2] + K[K_d33]*x[47], K[K_d35]*x[45] + het[4]*x[12] + tj[J_hocl]);
    const T D_r10 = nt_div<T>(K[K_d60]*x[52], F.hnm*K[K_d61] + tj[J_cl2o2]);
    const T D_r12 = nt_div<T>(K[K_e5c]*x[53], tj[J_brcl]);
    const T D_r11 = nt_div<T>(T(2)*D_r10*tj[J_cl2o2] + D_r12*tj[J_brcl] + D_r13*tj[J_clono2_cl] + D_r9*tj[J_hocl] + K[K_c18]*x[28] + K[K_d3]*x[45] + K[K_d4]*x[49] + K[K_d8]*x[43] + K[K_e5b]*x[53], K[K_d10]*x[47] + K[K_d2]*x[46] + K[K_d37]*x[14] + K[K_d5]*x[1] + K[K_d7]*x[47]);
    R[44] = -D_r11*x[52] + x[44];
    R[52] = nt_div<T>(-x[22], D_r11 + T(1)) + x[52];
    const T D_r27 = nt_div<T>(K[K_e13]*x[48], K[K_e8]*x[45] + tj[J_brono2]);
    const T D_r28 = nt_div<T>(K[K_e15]*x[47], K[K_e16]*x[45] + tj[J_hobr]);
    const T D_r29 = nt_div<T>(K[K_e5c]*x[52], tj[J_brcl]);
    const T D_r30 = nt_div<T>(T(0.85)*D_r27*tj[J_brono2] + D_r28*tj[J_hobr] + D_r29*tj[J_brcl] + K[K_e10]*x[43] + K[K_e3]*x[45] + K[K_e4]*x[49] + K[K_e5a]*x[52] + K[K_e5b]*x[52] + T(2)*K[K_e6]*x[53] + tj[J_bro], K[K_c19]*x[27] + K[K_e2]*x[46] + K[K_e7]*x[47]);
    R[50] = -D_r30*x[53] + x[50];
    R[53] = nt_div<T>(-x[23], D_r30 + T(1)) + x[53];
}

// scaled Jacobian rows [2, 7, 14, 19, 21, 23, 24, 26, 28, 32, 35, 37, 41, 44, 48, 49, 51, 54, 56] (day equations) into their stored A slots
template <typename T, typename FF, typename PK, typename PJ>
__device__ __forceinline__ void nt_jacobian_day_w4_3(const FF& F, PK K, PK tj, PK het, const double* __restrict__ x, double floor_, PJ J) {
    const int fh = nt_exp_hi(floor_);
    const T xt0 = nt_cvt<T>(x[0]);
    const T xt1 = nt_cvt<T>(x[1]);
    const T xt2 = nt_cvt<T>(x[2]);
    const T xt3 = nt_cvt<T>(x[3]);
    const T xt4 = nt_cvt<T>(x[4]);
    const T xt5 = nt_cvt<T>(x[5]);
    const T xt6 = nt_cvt<T>(x[6]);
    const T xt7 = nt_cvt<T>(x[7]);
    const T xt8 = nt_cvt<T>(x[8]);
    const T xt9 = nt_cvt<T>(x[9]);
    const T xt10 = nt_cvt<T>(x[10]);
    const T xt11 = nt_cvt<T>(x[11]);
    const T xt12 = nt_cvt<T>(x[12]);
    const T xt13 = nt_cvt<T>(x[13]);
    const T xt14 = nt_cvt<T>(x[14]);
    const T xt15 = nt_cvt<T>(x[15]);
    const T xt16 = nt_cvt<T>(x[16]);
    const T xt17 = nt_cvt<T>(x[17]);
    const T xt18 = nt_cvt<T>(x[18]);
    const T xt19 = nt_cvt<T>(x[19]);
    const T xt20 = nt_cvt<T>(x[20]);
    const T xt21 = nt_cvt<T>(x[21]);
    const T xt22 = nt_cvt<T>(x[22]);
    const T xt23 = nt_cvt<T>(x[23]);
    const T xt24 = nt_cvt<T>(x[24]);
    const T xt25 = nt_cvt<T>(x[25]);
    const T xt26 = nt_cvt<T>(x[26]);
    const T xt27 = nt_cvt<T>(x[27]);
    const T xt28 = nt_cvt<T>(x[28]);
    const T xt29 = nt_cvt<T>(x[29]);
    const T xt30 = nt_cvt<T>(x[30]);
    const T xt31 = nt_cvt<T>(x[31]);
    const T xt32 = nt_cvt<T>(x[32]);
    const T xt33 = nt_cvt<T>(x[33]);
    const T xt34 = nt_cvt<T>(x[34]);
    const T xt35 = nt_cvt<T>(x[35]);
    const T xt36 = nt_cvt<T>(x[36]);
    const T xt37 = nt_cvt<T>(x[37]);
    const T xt38 = nt_cvt<T>(x[38]);
    const T xt39 = nt_cvt<T>(x[39]);
    const T xt40 = nt_cvt<T>(x[40]);
    const T xt41 = nt_cvt<T>(x[41]);
    const T xt42 = nt_cvt<T>(x[42]);
    const T xt43 = nt_cvt<T>(x[43]);
    const T xt44 = nt_cvt<T>(x[44]);
    const T xt45 = nt_cvt<T>(x[45]);
    const T xt46 = nt_cvt<T>(x[46]);
    const T xt47 = nt_cvt<T>(x[47]);
    const T xt48 = nt_cvt<T>(x[48]);
    const T xt49 = nt_cvt<T>(x[49]);
    const T xt50 = nt_cvt<T>(x[50]);
    const T xt51 = nt_cvt<T>(x[51]);
    const T xt52 = nt_cvt<T>(x[52]);
    const T xt53 = nt_cvt<T>(x[53]);
    const T xt54 = nt_cvt<T>(x[54]);
    const T xt55 = nt_cvt<T>(x[55]);
    const T xt56 = nt_cvt<T>(x[56]);
    const T cs1 = nt_scale<T>(nt_exp_hi(x[1]), fh);
    const T cs2 = nt_scale<T>(nt_exp_hi(x[2]), fh);
    const T cs4 = nt_scale<T>(nt_exp_hi(x[4]), fh);
    const T cs12 = nt_scale<T>(nt_exp_hi(x[12]), fh);
    const T cs13 = nt_scale<T>(nt_exp_hi(x[13]), fh);
    const T cs14 = nt_scale<T>(nt_exp_hi(x[14]), fh);
    const T cs16 = nt_scale<T>(nt_exp_hi(x[16]), fh);
    const T cs18 = nt_scale<T>(nt_exp_hi(x[18]), fh);
    const T cs19 = nt_scale<T>(nt_exp_hi(x[19]), fh);
    const T cs20 = nt_scale<T>(nt_exp_hi(x[20]), fh);
    const T cs21 = nt_scale<T>(nt_exp_hi(x[21]), fh);
    const T cs24 = nt_scale<T>(nt_exp_hi(x[24]), fh);
    const T cs25 = nt_scale<T>(nt_exp_hi(x[25]), fh);
    const T cs26 = nt_scale<T>(nt_exp_hi(x[26]), fh);
    const T cs27 = nt_scale<T>(nt_exp_hi(x[27]), fh);
    const T cs28 = nt_scale<T>(nt_exp_hi(x[28]), fh);
    const T cs29 = nt_scale<T>(nt_exp_hi(x[29]), fh);
    const T cs32 = nt_scale<T>(nt_exp_hi(x[32]), fh);
    const T cs35 = nt_scale<T>(nt_exp_hi(x[35]), fh);
    const T cs37 = nt_scale<T>(nt_exp_hi(x[37]), fh);
    const T cs41 = nt_scale<T>(nt_exp_hi(x[41]), fh);
    const T cs42 = nt_scale<T>(nt_exp_hi(x[42]), fh);
    const T cs43 = nt_scale<T>(nt_exp_hi(x[43]), fh);
    const T cs44 = nt_scale<T>(nt_exp_hi(x[44]), fh);
    const T cs45 = nt_scale<T>(nt_exp_hi(x[45]), fh);
    const T cs46 = nt_scale<T>(nt_exp_hi(x[46]), fh);
    const T cs47 = nt_scale<T>(nt_exp_hi(x[47]), fh);
    const T cs48 = nt_scale<T>(nt_exp_hi(x[48]), fh);
    const T cs49 = nt_scale<T>(nt_exp_hi(x[49]), fh);
    const T cs50 = nt_scale<T>(nt_exp_hi(x[50]), fh);
    const T cs52 = nt_scale<T>(nt_exp_hi(x[52]), fh);
    const T cs53 = nt_scale<T>(nt_exp_hi(x[53]), fh);
    const T cs55 = nt_scale<T>(nt_exp_hi(x[55]), fh);
    const T cs56 = nt_scale<T>(nt_exp_hi(x[56]), fh);
    {  // row 2
    const T rs2 = nt_rscale<T>(nt_exp_hi(x[2]), fh);
        const T dj2_c0 = F.dt*xt43;
        const T dj2_c1 = F.dt*F.parth2o;
        const T dj2_c2 = F.parthno3*K[K_b27];
        const T dj2_c3 = F.parthcl*K[K_d11];
        J[261] = (-K[K_c2]*dj2_c0) * (cs1 * rs2);
        J[266] = (dj2_c1*(K[K_a1et]*xt42 + tj[J_h2o]) + T(1)) * (cs2 * rs2);
        J[260] = (-dj2_c0*dj2_c2) * (cs4 * rs2);
        J[265] = (-dj2_c0*dj2_c3) * (cs12 * rs2);
        J[262] = (-K[K_a30]*dj2_c0) * (cs16 * rs2);
        J[264] = (-K[K_c8]*dj2_c0) * (cs27 * rs2);
        J[258] = (-F.dt*(K[K_c17a]*xt43 + K[K_c17b]*xt43)) * (cs29 * rs2);
        J[259] = (K[K_a1et]*dj2_c1*xt2) * (cs42 * rs2);
        J[267] = (-F.dt*(F.h2*K[K_a19] + K[K_a17]*xt47 + K[K_a30]*xt16 + T(2)*K[K_a31]*xt43 + K[K_c17a]*xt29 + K[K_c17b]*xt29 + K[K_c2]*xt1 + K[K_c8]*xt27 + dj2_c2*xt4 + dj2_c3*xt12)) * (cs43 * rs2);
        J[268] = (-F.dt*(K[K_a17]*xt43 + T(1.6e-12)*xt55)) * (cs47 * rs2);
        J[263] = (-T(1.6e-12)*F.dt*xt47) * (cs55 * rs2);
    }
    {  // row 14
    const T rs14 = nt_rscale<T>(nt_exp_hi(x[14]), fh);
        const T dj14_c0 = F.dt*het[0];
        const T dj14_c1 = F.dt*xt14;
        const T dj14_c2 = F.dt*K[K_d33];
        J[170] = (-dj14_c0*xt13) * (cs2 * rs14);
        J[169] = (dj14_c1*het[4]) * (cs12 * rs14);
        J[166] = (-dj14_c0*xt2) * (cs13 * rs14);
        J[167] = (F.dt*(K[K_d34]*xt43 + K[K_d35]*xt45 + K[K_d37]*xt44 + het[4]*xt12 + het[8]*xt18 + tj[J_hocl]) + T(1)) * (cs14 * rs14);
        J[168] = (dj14_c1*het[8]) * (cs18 * rs14);
        J[173] = (K[K_d34]*dj14_c1) * (cs43 * rs14);
        J[172] = (K[K_d37]*dj14_c1) * (cs44 * rs14);
        J[171] = (K[K_d35]*dj14_c1) * (cs45 * rs14);
        J[174] = (-dj14_c2*xt52) * (cs47 * rs14);
        J[175] = (-dj14_c2*xt47) * (cs52 * rs14);
    }
    {  // row 19
    const T rs19 = nt_rscale<T>(nt_exp_hi(x[19]), fh);
        const T dj19_c0 = F.dt*xt19;
        const T dj19_c1 = F.dt*K[K_e13];
        J[56] = (dj19_c0*het[5]) * (cs2 * rs19);
        J[55] = (F.dt*(K[K_e8]*xt45 + het[5]*xt2 + tj[J_brono2]) + T(1)) * (cs19 * rs19);
        J[58] = (K[K_e8]*dj19_c0) * (cs45 * rs19);
        J[57] = (-dj19_c1*xt53) * (cs48 * rs19);
        J[59] = (-dj19_c1*xt48) * (cs53 * rs19);
    }
    {  // row 21
    const T rs21 = nt_rscale<T>(nt_exp_hi(x[21]), fh);
        const T dj21_c0 = F.dt*K[K_b23];
        J[152] = (F.dt*(F.hnm*K[K_b24] + K[K_b28]*xt43 + tj[J_hno4]) + T(1)) * (cs21 * rs21);
        J[154] = (F.dt*K[K_b28]*xt21) * (cs43 * rs21);
        J[155] = (-dj21_c0*xt48) * (cs47 * rs21);
        J[153] = (-dj21_c0*xt47) * (cs48 * rs21);
    }
    {  // row 23
    const T rs23 = nt_rscale<T>(nt_exp_hi(x[23]), fh);
        const T dj23_c0 = T(2)*het[7];
        const T dj23_c1 = F.dt*F.parthbr*xt18;
        const T dj23_c2 = F.dt*xt53;
        J[196] = (-F.dt*(F.parthbr*(K[K_e11]*xt43 + K[K_e9]*xt42 + tj[J_hbr]) + dj23_c0*xt25)) * (cs18 * rs23);
        J[193] = (-F.dt*(K[K_e8]*xt45 + tj[J_brono2])) * (cs19 * rs23);
        J[194] = (-F.dt*(K[K_e16]*xt45 + dj23_c0*xt18 + tj[J_hobr])) * (cs25 * rs23);
        J[192] = (-F.dt*tj[J_brcl]) * (cs26 * rs23);
        J[197] = (F.dt*K[K_c19]*xt50) * (cs27 * rs23);
        J[195] = (-K[K_e9]*dj23_c1) * (cs42 * rs23);
        J[202] = (-K[K_e11]*dj23_c1) * (cs43 * rs23);
        J[199] = (-F.dt*(K[K_e16]*xt25 + K[K_e8]*xt19)) * (cs45 * rs23);
        J[203] = (F.dt*(K[K_e15]*xt53 + K[K_e7]*xt50)) * (cs47 * rs23);
        J[198] = (K[K_e13]*dj23_c2) * (cs48 * rs23);
        J[201] = (F.dt*(K[K_c19]*xt27 + K[K_e7]*xt47)) * (cs50 * rs23);
        J[204] = (K[K_e5c]*dj23_c2) * (cs52 * rs23);
        J[200] = (F.dt*(K[K_e13]*xt48 + K[K_e15]*xt47 + K[K_e5c]*xt52)) * (cs53 * rs23);
    }
    {  // row 24
    const T rs24 = nt_rscale<T>(nt_exp_hi(x[24]), fh);
        J[97] = (F.dt*(F.hnm*K[K_d61] + tj[J_cl2o2]) + T(1)) * (cs24 * rs24);
        J[98] = (-T(2)*F.dt*K[K_d60]*xt52) * (cs52 * rs24);
    }
    {  // row 26
    const T rs26 = nt_rscale<T>(nt_exp_hi(x[26]), fh);
        const T dj26_c0 = F.dt*het[6];
        const T dj26_c1 = F.dt*het[8];
        const T dj26_c2 = F.dt*K[K_e5c];
        J[47] = (-dj26_c0*xt25) * (cs12 * rs26);
        J[45] = (-dj26_c1*xt18) * (cs14 * rs26);
        J[46] = (-dj26_c1*xt14) * (cs18 * rs26);
        J[44] = (-dj26_c0*xt12) * (cs25 * rs26);
        J[43] = (F.dt*tj[J_brcl] + T(1)) * (cs26 * rs26);
        J[49] = (-dj26_c2*xt53) * (cs52 * rs26);
        J[48] = (-dj26_c2*xt52) * (cs53 * rs26);
    }
    {  // row 28
    const T rs28 = nt_rscale<T>(nt_exp_hi(x[28]), fh);
        const T dj28_c0 = T(2)*K[K_c14]*xt28;
        const T dj28_c1 = F.dt*K[K_c17a];
        const T dj28_c2 = F.dt*xt28;
        J[212] = (F.dt*dj28_c0 + F.dt*(K[K_c18]*xt52 + K[K_c5]*xt49 + K[K_c7]*xt47 + dj28_c0) + T(1)) * (cs28 * rs28);
        J[210] = (-dj28_c1*xt43) * (cs29 * rs28);
        J[213] = (-dj28_c1*xt29) * (cs43 * rs28);
        J[214] = (K[K_c7]*dj28_c2) * (cs47 * rs28);
        J[215] = (K[K_c5]*dj28_c2) * (cs49 * rs28);
        J[216] = (K[K_c18]*dj28_c2) * (cs52 * rs28);
        J[211] = (-F.dt*F.o2*K[K_c4]) * (cs56 * rs28);
    }
    {  // row 32
    const T rs32 = nt_rscale<T>(nt_exp_hi(x[32]), fh);
        J[18] = (F.dt*(K[K_d92]*xt42 + tj[J_cfc113]) + T(1)) * (cs32 * rs32);
        J[19] = (F.dt*K[K_d92]*xt32) * (cs42 * rs32);
    }
    {  // row 35
    const T rs35 = nt_rscale<T>(nt_exp_hi(x[35]), fh);
        J[66] = (F.dt*(K[K_d95]*xt43 + tj[J_ch3cl]) + T(1)) * (cs35 * rs35);
        J[67] = (F.dt*K[K_d95]*xt35) * (cs43 * rs35);
    }
    {  // row 37
    const T rs37 = nt_rscale<T>(nt_exp_hi(x[37]), fh);
        const T dj37_c0 = F.dt*xt37;
        J[52] = (F.dt*(K[K_e50]*xt42 + K[K_e51]*xt43 + tj[J_ch3br]) + T(1)) * (cs37 * rs37);
        J[53] = (K[K_e50]*dj37_c0) * (cs42 * rs37);
        J[54] = (K[K_e51]*dj37_c0) * (cs43 * rs37);
    }
    {  // row 41
    const T rs41 = nt_rscale<T>(nt_exp_hi(x[41]), fh);
        J[125] = (F.dt*(K[K_e54]*xt43 + tj[J_ch2br2]) + T(1)) * (cs41 * rs41);
        J[126] = (F.dt*K[K_e54]*xt41) * (cs43 * rs41);
    }
    {  // row 56
    const T rs56 = nt_rscale<T>(nt_exp_hi(x[56]), fh);
        const T dj56_c0 = F.o2*K[K_c4] + K[K_c3]*xt45;
        const T dj56_c1 = nt_div<T>(T(1), dj56_c0);
        const T dj56_c2 = K[K_c1a]*xt42 + K[K_c2]*xt43 + K[K_d5]*xt44;
        const T dj56_c3 = dj56_c1*xt1;
        J[177] = (-dj56_c1*dj56_c2) * (cs1 * rs56);
        J[176] = (-K[K_c1a]*dj56_c3) * (cs42 * rs56);
        J[180] = (-K[K_c2]*dj56_c3) * (cs43 * rs56);
        J[179] = (-K[K_d5]*dj56_c3) * (cs44 * rs56);
        J[178] = (nt_div<T>(K[K_c3]*dj56_c2*xt1, (dj56_c0*dj56_c0))) * (cs45 * rs56);
    }
    const T D_r7_c0 = F.o2*K[K_b7] + K[K_b6]*xt49;
    const T D_r7 = nt_div<T>(tj[J_no], D_r7_c0);
    const T d_D_r7_49 = nt_div<T>(-K[K_b6]*tj[J_no], (D_r7_c0*D_r7_c0));
    {  // row 51
    const T rs51 = nt_rscale<T>(nt_exp_hi(x[51]), fh);
        J[78] = (-D_r7 - d_D_r7_49*xt49) * (cs49 * rs51);
    }
    const T D_r8_c0 = K[K_b12]*xt48 + tj[J_no3_no2] + tj[J_no3_no];
    const T D_r8_c1 = nt_div<T>(K[K_b9], D_r8_c0);
    const T D_r8 = D_r8_c1*xt46;
    const T d_D_r8_46 = D_r8_c1;
    const T d_D_r8_48 = nt_div<T>(-K[K_b12]*K[K_b9]*xt46, (D_r8_c0*D_r8_c0));
    {  // row 54
    const T rs54 = nt_rscale<T>(nt_exp_hi(x[54]), fh);
        J[68] = T(0);
        J[70] = (-d_D_r8_46*xt48) * (cs46 * rs54);
        J[69] = (-D_r8 - d_D_r8_48*xt48) * (cs48 * rs54);
    }
    const T D_r5_c0 = D_r8*tj[J_no3_no] + K[K_b3]*xt45 + tj[J_no2];
    const T D_r5_c1 = K[K_a26]*xt47 + K[K_b4]*xt46 + K[K_c5]*xt28 + K[K_d4]*xt52 + K[K_e4]*xt53;
    const T D_r5_c2 = nt_div<T>(T(1), D_r5_c1);
    const T D_r5_c3 = nt_div<T>(D_r5_c0, (D_r5_c1*D_r5_c1));
    const T D_r5 = D_r5_c0*D_r5_c2;
    const T d_D_r5_28 = -D_r5_c3*K[K_c5];
    const T d_D_r5_45 = D_r5_c2*K[K_b3];
    const T d_D_r5_46 = D_r5_c2*d_D_r8_46*tj[J_no3_no] - D_r5_c3*K[K_b4];
    const T d_D_r5_47 = -D_r5_c3*K[K_a26];
    const T d_D_r5_48 = D_r5_c2*d_D_r8_48*tj[J_no3_no];
    const T d_D_r5_52 = -D_r5_c3*K[K_d4];
    const T d_D_r5_53 = -D_r5_c3*K[K_e4];
    {  // row 48
    const T rs48 = nt_rscale<T>(nt_exp_hi(x[48]), fh);
        const T dj48_c0 = D_r5*D_r7 + D_r5 + D_r8 + T(1);
        const T dj48_c1 = nt_div<T>(T(1), dj48_c0*dj48_c0);
        const T dj48_c2 = dj48_c1*xt20;
        const T dj48_c3 = dj48_c2*(-D_r7 + T(-1));
        J[270] = (nt_div<T>(T(-1), dj48_c0)) * (cs20 * rs48);
        J[269] = (-d_D_r5_28*dj48_c3) * (cs28 * rs48);
        J[272] = (-d_D_r5_45*dj48_c3) * (cs45 * rs48);
        J[275] = (-d_D_r5_46*dj48_c3 + d_D_r8_46*dj48_c1*xt20) * (cs46 * rs48);
        J[274] = (-d_D_r5_47*dj48_c3) * (cs47 * rs48);
        J[271] = (-d_D_r5_48*dj48_c3 + d_D_r8_48*dj48_c2 + T(1)) * (cs48 * rs48);
        J[276] = (D_r5*d_D_r7_49*dj48_c2) * (cs49 * rs48);
        J[277] = (-d_D_r5_52*dj48_c3) * (cs52 * rs48);
        J[273] = (-d_D_r5_53*dj48_c3) * (cs53 * rs48);
    }
    {  // row 49
    const T rs49 = nt_rscale<T>(nt_exp_hi(x[49]), fh);
        J[361] = (-d_D_r5_28*xt48) * (cs28 * rs49);
        J[363] = (-d_D_r5_45*xt48) * (cs45 * rs49);
        J[366] = (-d_D_r5_46*xt48) * (cs46 * rs49);
        J[365] = (-d_D_r5_47*xt48) * (cs47 * rs49);
        J[362] = (-D_r5 - d_D_r5_48*xt48) * (cs48 * rs49);
        J[367] = (-d_D_r5_52*xt48) * (cs52 * rs49);
        J[364] = (-d_D_r5_53*xt48) * (cs53 * rs49);
    }
    const T D_r13_c0 = K[K_d32]*xt45 + het[0]*xt2 + het[1]*xt12 + tj[J_clono2_cl] + tj[J_clono2_clo];
    const T D_r13_c1 = nt_div<T>(K[K_d31], D_r13_c0);
    const T D_r13_c2 = nt_div<T>(K[K_d31]*xt48, (D_r13_c0*D_r13_c0));
    const T D_r13 = D_r13_c1*xt48;
    const T d_D_r13_2 = -D_r13_c2*het[0];
    const T d_D_r13_12 = -D_r13_c2*het[1];
    const T d_D_r13_45 = -D_r13_c2*K[K_d32];
    const T d_D_r13_48 = D_r13_c1;
    const T D_r9_c0 = D_r13*het[0];
    const T D_r9_c1 = D_r9_c0*xt2 + K[K_d33]*xt47;
    const T D_r9_c2 = K[K_d35]*xt45 + het[4]*xt12 + tj[J_hocl];
    const T D_r9_c3 = nt_div<T>(T(1), D_r9_c2);
    const T D_r9_c4 = D_r9_c3*het[0]*xt2;
    const T D_r9_c5 = nt_div<T>(D_r9_c1, (D_r9_c2*D_r9_c2));
    const T D_r9 = D_r9_c1*D_r9_c3;
    const T d_D_r9_2 = D_r9_c0*D_r9_c3 + D_r9_c4*d_D_r13_2;
    const T d_D_r9_12 = D_r9_c4*d_D_r13_12 - D_r9_c5*het[4];
    const T d_D_r9_45 = D_r9_c3*d_D_r13_45*het[0]*xt2 - D_r9_c5*K[K_d35];
    const T d_D_r9_47 = D_r9_c3*K[K_d33];
    const T d_D_r9_48 = D_r9_c4*d_D_r13_48;
    const T D_r10_c0 = nt_div<T>(K[K_d60], F.hnm*K[K_d61] + tj[J_cl2o2]);
    const T D_r10 = D_r10_c0*xt52;
    const T d_D_r10_52 = D_r10_c0;
    const T D_r12_c0 = nt_div<T>(K[K_e5c], tj[J_brcl]);
    const T D_r12 = D_r12_c0*xt53;
    const T d_D_r12_53 = D_r12_c0;
    const T D_r11_c0 = K[K_d10]*xt47 + K[K_d2]*xt46 + K[K_d37]*xt14 + K[K_d5]*xt1 + K[K_d7]*xt47;
    const T D_r11_c1 = nt_div<T>(T(1), D_r11_c0);
    const T D_r11_c2 = T(2)*tj[J_cl2o2];
    const T D_r11_c3 = D_r10*D_r11_c2 + D_r12*tj[J_brcl] + D_r13*tj[J_clono2_cl] + D_r9*tj[J_hocl] + K[K_c18]*xt28 + K[K_d3]*xt45 + K[K_d4]*xt49 + K[K_d8]*xt43 + K[K_e5b]*xt53;
    const T D_r11_c4 = nt_div<T>(D_r11_c3, (D_r11_c0*D_r11_c0));
    const T D_r11_c5 = D_r11_c1*tj[J_clono2_cl];
    const T D_r11_c6 = D_r11_c1*tj[J_hocl];
    const T D_r11 = D_r11_c1*D_r11_c3;
    const T d_D_r11_1 = -D_r11_c4*K[K_d5];
    const T d_D_r11_2 = D_r11_c5*d_D_r13_2 + D_r11_c6*d_D_r9_2;
    const T d_D_r11_12 = D_r11_c5*d_D_r13_12 + D_r11_c6*d_D_r9_12;
    const T d_D_r11_14 = -D_r11_c4*K[K_d37];
    const T d_D_r11_28 = D_r11_c1*K[K_c18];
    const T d_D_r11_43 = D_r11_c1*K[K_d8];
    const T d_D_r11_45 = D_r11_c1*K[K_d3] + D_r11_c5*d_D_r13_45 + D_r11_c6*d_D_r9_45;
    const T d_D_r11_46 = -D_r11_c4*K[K_d2];
    const T d_D_r11_47 = D_r11_c4*(-K[K_d10] - K[K_d7]) + D_r11_c6*d_D_r9_47;
    const T d_D_r11_48 = D_r11_c5*d_D_r13_48 + D_r11_c6*d_D_r9_48;
    const T d_D_r11_49 = D_r11_c1*K[K_d4];
    const T d_D_r11_52 = D_r11_c1*D_r11_c2*d_D_r10_52;
    const T d_D_r11_53 = D_r11_c1*K[K_e5b] + D_r11_c1*d_D_r12_53*tj[J_brcl];
    {  // row 44
    const T rs44 = nt_rscale<T>(nt_exp_hi(x[44]), fh);
        J[284] = (-d_D_r11_1*xt52) * (cs1 * rs44);
        J[288] = (-d_D_r11_2*xt52) * (cs2 * rs44);
        J[287] = (-d_D_r11_12*xt52) * (cs12 * rs44);
        J[285] = (-d_D_r11_14*xt52) * (cs14 * rs44);
        J[286] = (-d_D_r11_28*xt52) * (cs28 * rs44);
        J[292] = (-d_D_r11_43*xt52) * (cs43 * rs44);
        J[290] = (-d_D_r11_45*xt52) * (cs45 * rs44);
        J[294] = (-d_D_r11_46*xt52) * (cs46 * rs44);
        J[293] = (-d_D_r11_47*xt52) * (cs47 * rs44);
        J[289] = (-d_D_r11_48*xt52) * (cs48 * rs44);
        J[295] = (-d_D_r11_49*xt52) * (cs49 * rs44);
        J[296] = (-D_r11 - d_D_r11_52*xt52) * (cs52 * rs44);
        J[291] = (-d_D_r11_53*xt52) * (cs53 * rs44);
    }
    const T D_t06_c0 = tj[J_hocl]*xt14;
    const T D_t06_c1 = K[K_d33]*xt52;
    const T D_t06_c2 = D_t06_c1*xt47;
    const bool sel_D_t06 = (D_t06_c0) <= (D_t06_c2);
    const T D_t06 = sel_D_t06 ? T(D_t06_c0) : T(D_t06_c2);
    const T d_D_t06_14 = sel_D_t06 ? T(tj[J_hocl]) : T(T(0));
    const T d_D_t06_47 = sel_D_t06 ? T(T(0)) : T(D_t06_c1);
    const T d_D_t06_52 = sel_D_t06 ? T(T(0)) : T(K[K_d33]*xt47);
    const T D_t07_c0 = K[K_e5c]*xt53;
    const T D_t07_c1 = D_t07_c0*xt52;
    const T D_t07_c2 = tj[J_brcl]*xt26;
    const bool sel_D_t07 = (D_t07_c1) <= (D_t07_c2);
    const T D_t07 = sel_D_t07 ? T(D_t07_c1) : T(D_t07_c2);
    const T d_D_t07_26 = sel_D_t07 ? T(T(0)) : T(tj[J_brcl]);
    const T d_D_t07_52 = sel_D_t07 ? T(D_t07_c0) : T(T(0));
    const T d_D_t07_53 = sel_D_t07 ? T(K[K_e5c]*xt52) : T(T(0));
    const T D_t09_c0 = K[K_e15]*xt53;
    const T D_t09_c1 = D_t09_c0*xt47;
    const T D_t09_c2 = tj[J_hobr]*xt25;
    const bool sel_D_t09 = (D_t09_c1) <= (D_t09_c2);
    const T D_t09 = sel_D_t09 ? T(D_t09_c1) : T(D_t09_c2);
    const T d_D_t09_25 = sel_D_t09 ? T(T(0)) : T(tj[J_hobr]);
    const T d_D_t09_47 = sel_D_t09 ? T(D_t09_c0) : T(T(0));
    const T d_D_t09_53 = sel_D_t09 ? T(K[K_e15]*xt47) : T(T(0));
    {  // row 7
    const T rs7 = nt_rscale<T>(nt_exp_hi(x[7]), fh);
        const T dj7_c0 = T(2)*F.dt;
        const T dj7_c1 = nt_div<T>(tj[J_no3_no], fmax(T(1e-30), tj[J_no3_no2] + tj[J_no3_no]));
        const T dj7_c2 = F.dt*xt49;
        const T dj7_c3 = T(2)*K[K_b3];
        const T dj7_c4 = T(2)*K[K_d3];
        const T dj7_c5 = T(2)*K[K_hk3];
        const T dj7_c6 = T(2)*K[K_b9]*dj7_c1;
        const T dj7_c7 = T(2)*K[K_e5b];
        J[105] = (dj7_c0*dj7_c1*tj[J_clono2_cl]) * (cs13 * rs7);
        J[106] = (F.dt*d_D_t06_14) * (cs14 * rs7);
        J[104] = (F.dt*d_D_t09_25) * (cs25 * rs7);
        J[103] = (d_D_t07_26*dj7_c0) * (cs26 * rs7);
        J[108] = (-K[K_c5]*dj7_c2) * (cs28 * rs7);
        J[112] = (F.dt*(K[K_a5]*xt45 + K[K_a6]*xt46)) * (cs43 * rs7);
        J[110] = (F.dt*(K[K_a5]*xt43 + K[K_a7]*xt47 + T(4)*K[K_hk1]*xt45 + dj7_c3*xt48 + dj7_c4*xt52 + dj7_c5*xt46)) * (cs45 * rs7);
        J[114] = (F.dt*(K[K_a2]*xt55 + K[K_a6]*xt43 + K[K_a6b]*xt47 + dj7_c5*xt45 + dj7_c6*xt48)) * (cs46 * rs7);
        J[113] = (F.dt*d_D_t06_47 + F.dt*d_D_t09_47 + F.dt*(K[K_a6b]*xt46 + K[K_a7]*xt45) - K[K_a26]*dj7_c2) * (cs47 * rs7);
        J[109] = (F.dt*(dj7_c3*xt45 + dj7_c6*xt46)) * (cs48 * rs7);
        J[115] = (-F.dt*(K[K_a26]*xt47 + K[K_c5]*xt28)) * (cs49 * rs7);
        J[116] = (F.dt*d_D_t06_52 + F.dt*(nt_div<T>(T(4)*K[K_d60]*tj[J_cl2o2]*xt52, F.hnm*K[K_d61] + tj[J_cl2o2]) + dj7_c4*xt45 + dj7_c7*xt53) + d_D_t07_52*dj7_c0) * (cs52 * rs7);
        J[111] = (F.dt*d_D_t09_53 + F.dt*(T(4)*K[K_e6]*xt53 + dj7_c7*xt52) + d_D_t07_53*dj7_c0) * (cs53 * rs7);
        J[107] = (F.dt*K[K_a2]*xt46) * (cs55 * rs7);
    }
}

// residual rows of group g of 4 (day equations)
template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>
__device__ __forceinline__ void nt_residual_day_w4(int g, const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {
    switch (g) {
        case 0: nt_residual_day_w4_0<T>(F, K, tj, het, ck0, x, R); break;
        case 1: nt_residual_day_w4_1<T>(F, K, tj, het, ck0, x, R); break;
        case 2: nt_residual_day_w4_2<T>(F, K, tj, het, ck0, x, R); break;
        case 3: nt_residual_day_w4_3<T>(F, K, tj, het, ck0, x, R); break;
        default: break;
    }
}
// Jacobian rows of group g of 4 (day equations)
template <typename T, typename FF, typename PK, typename PJ>
__device__ __forceinline__ void nt_jacobian_day_w4(int g, const FF& F, PK K, PK tj, PK het, const double* __restrict__ x, double floor_, PJ J) {
    switch (g) {
        case 0: nt_jacobian_day_w4_0<T>(F, K, tj, het, x, floor_, J); break;
        case 1: nt_jacobian_day_w4_1<T>(F, K, tj, het, x, floor_, J); break;
        case 2: nt_jacobian_day_w4_2<T>(F, K, tj, het, x, floor_, J); break;
        case 3: nt_jacobian_day_w4_3<T>(F, K, tj, het, x, floor_, J); break;
        default: break;
    }
}

// residual R(x), night equations (FP64; K/tj/het/ck0/x: pointers or views)
template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>
__device__ __forceinline__ void nt_residual_night(const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {
    R[0] = -ck0[0] + x[0]*(F.dt*(tj[J_n2o] + x[42]*(K[K_b38] + K[K_b39])) + T(1));
    R[1] = -ck0[1] + x[1]*(F.dt*(K[K_c1a]*x[42] + K[K_c1b]*x[42] + K[K_c1c]*x[42] + K[K_c2]*x[43] + K[K_d5]*x[44]) + T(1));
    const T nr2_c0 = x[29]*x[43];
    R[2] = -F.dt*(F.h2*K[K_a19]*x[43] + F.parthcl*K[K_d11]*x[12]*x[43] + F.parthno3*K[K_b27]*x[43]*x[4] + K[K_a30]*x[16]*x[43] + K[K_a31]*(x[43]*x[43]) + K[K_c17a]*nr2_c0 + K[K_c17b]*nr2_c0 + K[K_c2]*x[1]*x[43] + K[K_c8]*x[27]*x[43] + x[47]*(K[K_a17]*x[43] + T(1.6e-12)*x[55])) - ck0[2] + x[2]*(F.dt*F.parth2o*(K[K_a1et]*x[42] + tj[J_h2o]) + T(1));
    R[3] = -T(2)*F.dt*K[K_b39]*x[0]*x[42] + F.dt*(F.rain_hno3*x[4] + T(2)*K[K_b6]*x[49]*x[51]) - ck0[3] + x[3];
    R[4] = -F.dt*(K[K_b22]*x[43]*x[48] + het[0]*x[13]*x[2] + het[1]*x[12]*x[13] + T(2)*het[2]*x[2]*x[5] + het[3]*x[12]*x[5] + het[5]*x[19]*x[2]) - ck0[4] + x[4]*(F.dt*(F.parthno3*(K[K_b27]*x[43] + tj[J_hno3]) + F.rain_hno3) + T(1));
    R[5] = -F.dt*K[K_b12]*x[48]*x[54] - ck0[5] + x[5]*(F.dt*(F.hnm*K[K_b32] + het[2]*x[2] + het[3]*x[12] + tj[J_n2o5]) + T(1));
    const T nr6_c0 = T(3)*x[42];
    R[6] = F.dt*F.rain_hcl*x[12] - F.dt*(x[30]*(K[K_d90]*nr6_c0 + T(3)*tj[J_cfc11]) + x[31]*(T(2)*K[K_d91]*x[42] + T(2)*tj[J_cfc12]) + x[32]*(K[K_d92]*nr6_c0 + T(3)*tj[J_cfc113]) + x[33]*(T(4)*K[K_d93]*x[42] + T(4)*tj[J_ccl4]) + x[34]*(T(3)*K[K_d94]*x[43] + T(3)*tj[J_ch3ccl3]) + x[35]*(K[K_d95]*x[43] + tj[J_ch3cl]) + x[36]*(K[K_d96]*x[42] + K[K_d97]*x[43] + tj[J_hcfc22]) + x[38]*(K[K_e52]*x[42] + tj[J_h1211])) - ck0[6] + x[6];
    R[8] = -F.dt*(F.co2*tj[J_co2] + tj[J_ch2o_co]*x[27]) - ck0[8] + x[8]*(F.dt*K[K_a36]*x[43] + T(1));
    R[9] = -F.dt*K[K_e5a]*x[52]*x[53] - ck0[9] + x[9]*(F.dt*tj[J_oclo] + T(1));
    R[10] = -ck0[10] + x[10];
    R[11] = -ck0[11] + x[11];
    R[12] = -F.dt*(K[K_d9]*x[43]*x[52] + x[44]*(F.h2*K[K_d6] + K[K_c10]*x[27] + K[K_d5]*x[1] + K[K_d7]*x[47])) - ck0[12] + x[12]*(F.dt*(F.parthcl*(K[K_d11]*x[43] + tj[J_hcl]) + F.rain_hcl + het[1]*x[13] + het[3]*x[5] + het[4]*x[14] + het[6]*x[25]) + T(1));
    R[13] = -F.dt*K[K_d31]*x[48]*x[52] - ck0[13] + x[13]*(F.dt*(K[K_d32]*x[45] + het[0]*x[2] + het[1]*x[12] + tj[J_clono2_cl] + tj[J_clono2_clo]) + T(1));
    R[14] = -F.dt*(K[K_d33]*x[47]*x[52] + het[0]*x[13]*x[2]) - ck0[14] + x[14]*(F.dt*(K[K_d34]*x[43] + K[K_d35]*x[45] + K[K_d37]*x[44] + het[4]*x[12] + het[8]*x[18] + tj[J_hocl]) + T(1));
    R[15] = -F.dt*(K[K_d37]*x[14]*x[44] + K[K_d62]*(x[52]*x[52]) + het[1]*x[12]*x[13] + het[4]*x[12]*x[14]) - ck0[15] + x[15]*(F.dt*tj[J_cl2] + T(1));
    R[16] = -F.dt*K[K_a27]*(x[47]*x[47]) - ck0[16] + x[16]*(F.dt*(F.rain_h2o2 + K[K_a30]*x[43] + tj[J_h2o2]) + T(1));
    R[17] = -F.dt*(K[K_d36]*x[44]*x[48] + het[3]*x[12]*x[5]) - ck0[17] + x[17]*(F.dt*tj[J_clno2] + T(1));
    R[18] = -F.dt*(K[K_c19]*x[27]*x[50] + K[K_e7]*x[47]*x[50]) - ck0[18] + x[18]*(F.dt*(F.parthbr*(K[K_e11]*x[43] + K[K_e9]*x[42] + tj[J_hbr]) + F.rain_hbr + het[7]*x[25] + het[8]*x[14]) + T(1));
    R[19] = -F.dt*K[K_e13]*x[48]*x[53] - ck0[19] + x[19]*(F.dt*(K[K_e8]*x[45] + het[5]*x[2] + tj[J_brono2]) + T(1));
    const T nr20_c0 = F.parthno3*x[4];
    R[20] = F.dt*(T(2)*K[K_b6]*x[49]*x[51] + x[48]*(T(2)*K[K_b12]*x[54] + K[K_b22]*x[43] + K[K_b23]*x[47] + K[K_d31]*x[52] + K[K_d36]*x[44] + K[K_e13]*x[53])) - F.dt*(K[K_b27]*nr20_c0*x[43] + T(2)*K[K_b39]*x[0]*x[42] + K[K_d32]*x[13]*x[45] + K[K_e8]*x[19]*x[45] + nr20_c0*tj[J_hno3] + tj[J_brono2]*x[19] + tj[J_clno2]*x[17] + x[13]*(tj[J_clono2_cl] + tj[J_clono2_clo]) + x[21]*(F.hnm*K[K_b24] + K[K_b28]*x[43] + tj[J_hno4]) + x[5]*(T(2)*F.hnm*K[K_b32] + T(2)*tj[J_n2o5])) - ck0[20] + x[20];
    R[21] = -F.dt*K[K_b23]*x[47]*x[48] - ck0[21] + x[21]*(F.dt*(F.hnm*K[K_b24] + K[K_b28]*x[43] + tj[J_hno4]) + T(1));
    const T nr22_c0 = T(2)*x[52];
    const T nr22_c1 = T(3)*x[42];
    R[22] = F.dt*(x[44]*(F.h2*K[K_d6] + K[K_c10]*x[27] + K[K_d36]*x[48] + K[K_d37]*x[14] + K[K_d5]*x[1] + K[K_d7]*x[47]) + x[52]*(K[K_d31]*x[48] + K[K_d33]*x[47] + K[K_d60]*nr22_c0 + K[K_d62]*nr22_c0 + K[K_d9]*x[43] + K[K_e5a]*x[53] + K[K_e5c]*x[53])) - F.dt*(F.parthcl*x[12]*(K[K_d11]*x[43] + tj[J_hcl]) + tj[J_brcl]*x[26] + T(2)*tj[J_cl2]*x[15] + tj[J_clno2]*x[17] + tj[J_oclo]*x[9] + x[13]*(K[K_d32]*x[45] + tj[J_clono2_cl] + tj[J_clono2_clo]) + x[14]*(K[K_d34]*x[43] + K[K_d35]*x[45] + tj[J_hocl]) + x[24]*(T(2)*F.hnm*K[K_d61] + T(2)*tj[J_cl2o2]) + x[30]*(K[K_d90]*nr22_c1 + T(3)*tj[J_cfc11]) + x[31]*(T(2)*K[K_d91]*x[42] + T(2)*tj[J_cfc12]) + x[32]*(K[K_d92]*nr22_c1 + T(3)*tj[J_cfc113]) + x[33]*(T(4)*K[K_d93]*x[42] + T(4)*tj[J_ccl4]) + x[34]*(T(3)*K[K_d94]*x[43] + T(3)*tj[J_ch3ccl3]) + x[35]*(K[K_d95]*x[43] + tj[J_ch3cl]) + x[36]*(K[K_d96]*x[42] + K[K_d97]*x[43] + tj[J_hcfc22])) - ck0[22] + x[22];
    R[23] = F.dt*(K[K_c19]*x[27]*x[50] + K[K_e7]*x[47]*x[50] + x[53]*(K[K_e13]*x[48] + K[K_e15]*x[47] + K[K_e5c]*x[52])) - F.dt*(F.parthbr*x[18]*(K[K_e11]*x[43] + K[K_e9]*x[42] + tj[J_hbr]) + K[K_e16]*x[25]*x[45] + K[K_e8]*x[19]*x[45] + T(2)*het[7]*x[18]*x[25] + tj[J_brcl]*x[26] + tj[J_brono2]*x[19] + tj[J_hobr]*x[25]) - ck0[23] + x[23];
    R[24] = -F.dt*K[K_d60]*(x[52]*x[52]) - ck0[24] + x[24]*(F.dt*(F.hnm*K[K_d61] + tj[J_cl2o2]) + T(1));
    R[25] = -F.dt*(K[K_e15]*x[47]*x[53] + het[5]*x[19]*x[2]) - ck0[25] + x[25]*(F.dt*(K[K_e16]*x[45] + het[6]*x[12] + het[7]*x[18] + tj[J_hobr]) + T(1));
    R[26] = -F.dt*(K[K_e5c]*x[52]*x[53] + het[6]*x[12]*x[25] + het[8]*x[14]*x[18]) - ck0[26] + x[26]*(F.dt*tj[J_brcl] + T(1));
    R[27] = -F.dt*(K[K_c17b]*x[29]*x[43] + K[K_c1c]*x[1]*x[42] + K[K_c3]*x[45]*x[56]) - ck0[27] + x[27]*(F.dt*(K[K_c10]*x[44] + K[K_c19]*x[50] + K[K_c8]*x[43] + K[K_c9]*x[45] + tj[J_ch2o_co] + tj[J_ch2o_hco]) + T(1));
    R[28] = -F.dt*(F.o2*K[K_c4]*x[56] + K[K_c17a]*x[29]*x[43]) - ck0[28] + x[28]*(F.dt*(T(2)*K[K_c14]*x[28] + K[K_c18]*x[52] + K[K_c5]*x[49] + K[K_c7]*x[47]) + T(1));
    R[29] = -F.dt*K[K_c7]*x[28]*x[47] - ck0[29] + x[29]*(F.dt*(K[K_c17a]*x[43] + K[K_c17b]*x[43] + tj[J_ch3o2h]) + T(1));
    R[30] = -ck0[30] + x[30]*(F.dt*(K[K_d90]*x[42] + tj[J_cfc11]) + T(1));
    R[31] = -ck0[31] + x[31]*(F.dt*(K[K_d91]*x[42] + tj[J_cfc12]) + T(1));
    R[32] = -ck0[32] + x[32]*(F.dt*(K[K_d92]*x[42] + tj[J_cfc113]) + T(1));
    R[33] = -ck0[33] + x[33]*(F.dt*(K[K_d93]*x[42] + tj[J_ccl4]) + T(1));
    R[34] = -ck0[34] + x[34]*(F.dt*(K[K_d94]*x[43] + tj[J_ch3ccl3]) + T(1));
    R[35] = -ck0[35] + x[35]*(F.dt*(K[K_d95]*x[43] + tj[J_ch3cl]) + T(1));
    R[36] = -ck0[36] + x[36]*(F.dt*(K[K_d96]*x[42] + K[K_d97]*x[43] + tj[J_hcfc22]) + T(1));
    R[37] = -ck0[37] + x[37]*(F.dt*(K[K_e50]*x[42] + K[K_e51]*x[43] + tj[J_ch3br]) + T(1));
    R[38] = -ck0[38] + x[38]*(F.dt*(K[K_e52]*x[42] + tj[J_h1211]) + T(1));
    R[39] = -ck0[39] + x[39]*(F.dt*(K[K_e53]*x[42] + tj[J_h1301]) + T(1));
    R[40] = F.dt*F.rain_hbr*x[18] - F.dt*(x[37]*(K[K_e50]*x[42] + K[K_e51]*x[43] + tj[J_ch3br]) + x[38]*(K[K_e52]*x[42] + tj[J_h1211]) + x[39]*(K[K_e53]*x[42] + tj[J_h1301]) + x[41]*(T(2)*K[K_e54]*x[43] + T(2)*tj[J_ch2br2])) - ck0[40] + x[40];
    R[41] = -ck0[41] + x[41]*(F.dt*(K[K_e54]*x[43] + tj[J_ch2br2]) + T(1));
    R[42] = x[42];
    R[43] = x[43];
    R[44] = x[44];
    R[45] = x[45];
    R[46] = x[46] - x[7];
    R[47] = x[47];
    R[49] = x[49];
    R[50] = x[50];
    R[51] = x[51];
    R[55] = x[55];
    R[56] = x[56];
    const T N_cno = nt_div<T>(K[K_b9]*x[46], K[K_b12]);
    const T N_dno = -N_cno + x[20];
    const bool sel_N_no2 = (N_dno) > (T(1e-30));
    const T N_no2 = sel_N_no2 ? T(N_dno) : T(nt_div<T>(T(1e-30)*x[20], N_cno + T(1e-30)));
    R[48] = -N_no2 + x[48];
    const bool sel_N_no3 = (N_dno) > (T(1e-30));
    const T N_no3 = sel_N_no3 ? T(N_cno) : T(nt_div<T>(N_cno*x[20], N_cno + T(1e-30)));
    R[54] = -N_no3 + x[54];
    const bool sel_N_clo = (x[22]) >= (T(0));
    const T N_clo = sel_N_clo ? T(x[22]) : T(T(0));
    R[52] = -N_clo + x[52];
    const bool sel_N_bro = (x[23]) >= (T(0));
    const T N_bro = sel_N_bro ? T(x[23]) : T(T(0));
    R[53] = -N_bro + x[53];
    const T N_t06_c0 = tj[J_hocl]*x[14];
    const T N_t06_c1 = K[K_d33]*x[47]*x[52];
    const bool sel_N_t06 = (N_t06_c0) <= (N_t06_c1);
    const T N_t06 = sel_N_t06 ? T(N_t06_c0) : T(N_t06_c1);
    const T N_t07_c0 = K[K_e5c]*x[52]*x[53];
    const T N_t07_c1 = tj[J_brcl]*x[26];
    const bool sel_N_t07 = (N_t07_c0) <= (N_t07_c1);
    const T N_t07 = sel_N_t07 ? T(N_t07_c0) : T(N_t07_c1);
    const T N_t09_c0 = K[K_e15]*x[47]*x[53];
    const T N_t09_c1 = tj[J_hobr]*x[25];
    const bool sel_N_t09 = (N_t09_c0) <= (N_t09_c1);
    const T N_t09 = sel_N_t09 ? T(N_t09_c0) : T(N_t09_c1);
    const T nr7_c0 = T(2)*x[45];
    const T nr7_c1 = nt_div<T>(T(2)*tj[J_no3_no], fmax(T(1e-30), tj[J_no3_no2] + tj[J_no3_no]));
    R[7] = -F.dt*(T(2)*F.o2*tj[J_o2] + K[K_a26]*x[47]*x[49] + K[K_c5]*x[28]*x[49]) + F.dt*(K[K_b3]*nr7_c0*x[48] + K[K_b9]*nr7_c1*x[46]*x[48] + K[K_d3]*nr7_c0*x[52] + nt_div<T>(T(2)*K[K_d60]*tj[J_cl2o2]*(x[52]*x[52]), F.hnm*K[K_d61] + tj[J_cl2o2]) + T(2)*K[K_hk1]*(x[45]*x[45]) + K[K_hk3]*nr7_c0*x[46] + N_t06 + T(2)*N_t07 + N_t09 + nr7_c1*tj[J_clono2_cl]*x[13] + x[45]*(K[K_a5]*x[43] + K[K_a7]*x[47]) + x[46]*(K[K_a2]*x[55] + K[K_a6]*x[43] + K[K_a6b]*x[47])) - ck0[7] + x[7];
}

// scaled Jacobian J'_ij = dR_i/dx_j s_j / s_i, night equations, into the
// stored A slots (T = double or float; x: FP64 iterate; s: nt_exp_hi scales)
template <typename T, typename FF, typename PK, typename PJ>
__device__ __forceinline__ void nt_jacobian_night(const FF& F, PK K, PK tj, PK het, const double* __restrict__ x, double floor_, PJ J) {
    const int fh = nt_exp_hi(floor_);
    // the iterate in T and the column scales, once per call
    const T xt0 = nt_cvt<T>(x[0]);
    const T xt1 = nt_cvt<T>(x[1]);
    const T xt2 = nt_cvt<T>(x[2]);
    const T xt3 = nt_cvt<T>(x[3]);
    const T xt4 = nt_cvt<T>(x[4]);
    const T xt5 = nt_cvt<T>(x[5]);
    const T xt6 = nt_cvt<T>(x[6]);
    const T xt7 = nt_cvt<T>(x[7]);
    const T xt8 = nt_cvt<T>(x[8]);
    const T xt9 = nt_cvt<T>(x[9]);
    const T xt10 = nt_cvt<T>(x[10]);
    const T xt11 = nt_cvt<T>(x[11]);
    const T xt12 = nt_cvt<T>(x[12]);
    const T xt13 = nt_cvt<T>(x[13]);
    const T xt14 = nt_cvt<T>(x[14]);
    const T xt15 = nt_cvt<T>(x[15]);
    const T xt16 = nt_cvt<T>(x[16]);
    const T xt17 = nt_cvt<T>(x[17]);
    const T xt18 = nt_cvt<T>(x[18]);
    const T xt19 = nt_cvt<T>(x[19]);
    const T xt20 = nt_cvt<T>(x[20]);
    const T xt21 = nt_cvt<T>(x[21]);
    const T xt22 = nt_cvt<T>(x[22]);
    const T xt23 = nt_cvt<T>(x[23]);
    const T xt24 = nt_cvt<T>(x[24]);
    const T xt25 = nt_cvt<T>(x[25]);
    const T xt26 = nt_cvt<T>(x[26]);
    const T xt27 = nt_cvt<T>(x[27]);
    const T xt28 = nt_cvt<T>(x[28]);
    const T xt29 = nt_cvt<T>(x[29]);
    const T xt30 = nt_cvt<T>(x[30]);
    const T xt31 = nt_cvt<T>(x[31]);
    const T xt32 = nt_cvt<T>(x[32]);
    const T xt33 = nt_cvt<T>(x[33]);
    const T xt34 = nt_cvt<T>(x[34]);
    const T xt35 = nt_cvt<T>(x[35]);
    const T xt36 = nt_cvt<T>(x[36]);
    const T xt37 = nt_cvt<T>(x[37]);
    const T xt38 = nt_cvt<T>(x[38]);
    const T xt39 = nt_cvt<T>(x[39]);
    const T xt40 = nt_cvt<T>(x[40]);
    const T xt41 = nt_cvt<T>(x[41]);
    const T xt42 = nt_cvt<T>(x[42]);
    const T xt43 = nt_cvt<T>(x[43]);
    const T xt44 = nt_cvt<T>(x[44]);
    const T xt45 = nt_cvt<T>(x[45]);
    const T xt46 = nt_cvt<T>(x[46]);
    const T xt47 = nt_cvt<T>(x[47]);
    const T xt48 = nt_cvt<T>(x[48]);
    const T xt49 = nt_cvt<T>(x[49]);
    const T xt50 = nt_cvt<T>(x[50]);
    const T xt51 = nt_cvt<T>(x[51]);
    const T xt52 = nt_cvt<T>(x[52]);
    const T xt53 = nt_cvt<T>(x[53]);
    const T xt54 = nt_cvt<T>(x[54]);
    const T xt55 = nt_cvt<T>(x[55]);
    const T xt56 = nt_cvt<T>(x[56]);
    const T cs0 = nt_scale<T>(nt_exp_hi(x[0]), fh);
    const T cs1 = nt_scale<T>(nt_exp_hi(x[1]), fh);
    const T cs2 = nt_scale<T>(nt_exp_hi(x[2]), fh);
    const T cs3 = nt_scale<T>(nt_exp_hi(x[3]), fh);
    const T cs4 = nt_scale<T>(nt_exp_hi(x[4]), fh);
    const T cs5 = nt_scale<T>(nt_exp_hi(x[5]), fh);
    const T cs6 = nt_scale<T>(nt_exp_hi(x[6]), fh);
    const T cs7 = nt_scale<T>(nt_exp_hi(x[7]), fh);
    const T cs8 = nt_scale<T>(nt_exp_hi(x[8]), fh);
    const T cs9 = nt_scale<T>(nt_exp_hi(x[9]), fh);
    const T cs10 = nt_scale<T>(nt_exp_hi(x[10]), fh);
    const T cs11 = nt_scale<T>(nt_exp_hi(x[11]), fh);
    const T cs12 = nt_scale<T>(nt_exp_hi(x[12]), fh);
    const T cs13 = nt_scale<T>(nt_exp_hi(x[13]), fh);
    const T cs14 = nt_scale<T>(nt_exp_hi(x[14]), fh);
    const T cs15 = nt_scale<T>(nt_exp_hi(x[15]), fh);
    const T cs16 = nt_scale<T>(nt_exp_hi(x[16]), fh);
    const T cs17 = nt_scale<T>(nt_exp_hi(x[17]), fh);
    const T cs18 = nt_scale<T>(nt_exp_hi(x[18]), fh);
    const T cs19 = nt_scale<T>(nt_exp_hi(x[19]), fh);
    const T cs20 = nt_scale<T>(nt_exp_hi(x[20]), fh);
    const T cs21 = nt_scale<T>(nt_exp_hi(x[21]), fh);
    const T cs22 = nt_scale<T>(nt_exp_hi(x[22]), fh);
    const T cs23 = nt_scale<T>(nt_exp_hi(x[23]), fh);
    const T cs24 = nt_scale<T>(nt_exp_hi(x[24]), fh);
    const T cs25 = nt_scale<T>(nt_exp_hi(x[25]), fh);
    const T cs26 = nt_scale<T>(nt_exp_hi(x[26]), fh);
    const T cs27 = nt_scale<T>(nt_exp_hi(x[27]), fh);
    const T cs28 = nt_scale<T>(nt_exp_hi(x[28]), fh);
    const T cs29 = nt_scale<T>(nt_exp_hi(x[29]), fh);
    const T cs30 = nt_scale<T>(nt_exp_hi(x[30]), fh);
    const T cs31 = nt_scale<T>(nt_exp_hi(x[31]), fh);
    const T cs32 = nt_scale<T>(nt_exp_hi(x[32]), fh);
    const T cs33 = nt_scale<T>(nt_exp_hi(x[33]), fh);
    const T cs34 = nt_scale<T>(nt_exp_hi(x[34]), fh);
    const T cs35 = nt_scale<T>(nt_exp_hi(x[35]), fh);
    const T cs36 = nt_scale<T>(nt_exp_hi(x[36]), fh);
    const T cs37 = nt_scale<T>(nt_exp_hi(x[37]), fh);
    const T cs38 = nt_scale<T>(nt_exp_hi(x[38]), fh);
    const T cs39 = nt_scale<T>(nt_exp_hi(x[39]), fh);
    const T cs40 = nt_scale<T>(nt_exp_hi(x[40]), fh);
    const T cs41 = nt_scale<T>(nt_exp_hi(x[41]), fh);
    const T cs42 = nt_scale<T>(nt_exp_hi(x[42]), fh);
    const T cs43 = nt_scale<T>(nt_exp_hi(x[43]), fh);
    const T cs44 = nt_scale<T>(nt_exp_hi(x[44]), fh);
    const T cs45 = nt_scale<T>(nt_exp_hi(x[45]), fh);
    const T cs46 = nt_scale<T>(nt_exp_hi(x[46]), fh);
    const T cs47 = nt_scale<T>(nt_exp_hi(x[47]), fh);
    const T cs48 = nt_scale<T>(nt_exp_hi(x[48]), fh);
    const T cs49 = nt_scale<T>(nt_exp_hi(x[49]), fh);
    const T cs50 = nt_scale<T>(nt_exp_hi(x[50]), fh);
    const T cs51 = nt_scale<T>(nt_exp_hi(x[51]), fh);
    const T cs52 = nt_scale<T>(nt_exp_hi(x[52]), fh);
    const T cs53 = nt_scale<T>(nt_exp_hi(x[53]), fh);
    const T cs54 = nt_scale<T>(nt_exp_hi(x[54]), fh);
    const T cs55 = nt_scale<T>(nt_exp_hi(x[55]), fh);
    const T cs56 = nt_scale<T>(nt_exp_hi(x[56]), fh);
    {  // row 0
    const T rs0 = nt_rscale<T>(nt_exp_hi(x[0]), fh);
        const T nj0_c0 = K[K_b38] + K[K_b39];
        J[76] = (F.dt*(nj0_c0*xt42 + tj[J_n2o]) + T(1)) * (cs0 * rs0);
        J[77] = (F.dt*nj0_c0*xt0) * (cs42 * rs0);
    }
    {  // row 1
    const T rs1 = nt_rscale<T>(nt_exp_hi(x[1]), fh);
        const T nj1_c0 = F.dt*xt1;
        J[157] = (F.dt*(K[K_c1a]*xt42 + K[K_c1b]*xt42 + K[K_c1c]*xt42 + K[K_c2]*xt43 + K[K_d5]*xt44) + T(1)) * (cs1 * rs1);
        J[156] = (nj1_c0*(K[K_c1a] + K[K_c1b] + K[K_c1c])) * (cs42 * rs1);
        J[159] = (K[K_c2]*nj1_c0) * (cs43 * rs1);
        J[158] = (K[K_d5]*nj1_c0) * (cs44 * rs1);
    }
    {  // row 2
    const T rs2 = nt_rscale<T>(nt_exp_hi(x[2]), fh);
        const T nj2_c0 = F.dt*xt43;
        const T nj2_c1 = F.dt*F.parth2o;
        const T nj2_c2 = F.parthno3*K[K_b27];
        const T nj2_c3 = F.parthcl*K[K_d11];
        J[261] = (-K[K_c2]*nj2_c0) * (cs1 * rs2);
        J[266] = (nj2_c1*(K[K_a1et]*xt42 + tj[J_h2o]) + T(1)) * (cs2 * rs2);
        J[260] = (-nj2_c0*nj2_c2) * (cs4 * rs2);
        J[265] = (-nj2_c0*nj2_c3) * (cs12 * rs2);
        J[262] = (-K[K_a30]*nj2_c0) * (cs16 * rs2);
        J[264] = (-K[K_c8]*nj2_c0) * (cs27 * rs2);
        J[258] = (-F.dt*(K[K_c17a]*xt43 + K[K_c17b]*xt43)) * (cs29 * rs2);
        J[259] = (K[K_a1et]*nj2_c1*xt2) * (cs42 * rs2);
        J[267] = (-F.dt*(F.h2*K[K_a19] + K[K_a17]*xt47 + K[K_a30]*xt16 + T(2)*K[K_a31]*xt43 + K[K_c17a]*xt29 + K[K_c17b]*xt29 + K[K_c2]*xt1 + K[K_c8]*xt27 + nj2_c2*xt4 + nj2_c3*xt12)) * (cs43 * rs2);
        J[268] = (-F.dt*(K[K_a17]*xt43 + T(1.6e-12)*xt55)) * (cs47 * rs2);
        J[263] = (-T(1.6e-12)*F.dt*xt47) * (cs55 * rs2);
    }
    {  // row 3
    const T rs3 = nt_rscale<T>(nt_exp_hi(x[3]), fh);
        const T nj3_c0 = T(2)*F.dt;
        const T nj3_c1 = K[K_b39]*nj3_c0;
        const T nj3_c2 = K[K_b6]*nj3_c0;
        J[20] = (-nj3_c1*xt42) * (cs0 * rs3);
        J[23] = (F.dt*F.rain_hno3) * (cs4 * rs3);
        J[22] = (-nj3_c1*xt0) * (cs42 * rs3);
        J[24] = (nj3_c2*xt51) * (cs49 * rs3);
        J[21] = (nj3_c2*xt49) * (cs51 * rs3);
    }
    {  // row 4
    const T rs4 = nt_rscale<T>(nt_exp_hi(x[4]), fh);
        const T nj4_c0 = T(2)*het[2];
        const T nj4_c1 = F.dt*K[K_b22];
        J[122] = (-F.dt*(het[0]*xt13 + het[5]*xt19 + nj4_c0*xt5)) * (cs2 * rs4);
        J[120] = (F.dt*(F.parthno3*(K[K_b27]*xt43 + tj[J_hno3]) + F.rain_hno3) + T(1)) * (cs4 * rs4);
        J[118] = (-F.dt*(het[3]*xt12 + nj4_c0*xt2)) * (cs5 * rs4);
        J[121] = (-F.dt*(het[1]*xt13 + het[3]*xt5)) * (cs12 * rs4);
        J[119] = (-F.dt*(het[0]*xt2 + het[1]*xt12)) * (cs13 * rs4);
        J[117] = (-F.dt*het[5]*xt2) * (cs19 * rs4);
        J[124] = (F.dt*F.parthno3*K[K_b27]*xt4 - nj4_c1*xt48) * (cs43 * rs4);
        J[123] = (-nj4_c1*xt43) * (cs48 * rs4);
    }
    {  // row 5
    const T rs5 = nt_rscale<T>(nt_exp_hi(x[5]), fh);
        const T nj5_c0 = F.dt*xt5;
        const T nj5_c1 = F.dt*K[K_b12];
        J[74] = (het[2]*nj5_c0) * (cs2 * rs5);
        J[72] = (F.dt*(F.hnm*K[K_b32] + het[2]*xt2 + het[3]*xt12 + tj[J_n2o5]) + T(1)) * (cs5 * rs5);
        J[73] = (het[3]*nj5_c0) * (cs12 * rs5);
        J[75] = (-nj5_c1*xt54) * (cs48 * rs5);
        J[71] = (-nj5_c1*xt48) * (cs54 * rs5);
    }
    {  // row 6
    const T rs6 = nt_rscale<T>(nt_exp_hi(x[6]), fh);
        const T nj6_c0 = T(3)*xt42;
        const T nj6_c1 = T(2)*K[K_d91];
        const T nj6_c2 = T(4)*K[K_d93];
        const T nj6_c3 = T(3)*K[K_d94];
        J[9] = (F.dt*F.rain_hcl) * (cs12 * rs6);
        J[7] = (-F.dt*(K[K_d90]*nj6_c0 + T(3)*tj[J_cfc11])) * (cs30 * rs6);
        J[4] = (-F.dt*(nj6_c1*xt42 + T(2)*tj[J_cfc12])) * (cs31 * rs6);
        J[0] = (-F.dt*(K[K_d92]*nj6_c0 + T(3)*tj[J_cfc113])) * (cs32 * rs6);
        J[2] = (-F.dt*(nj6_c2*xt42 + T(4)*tj[J_ccl4])) * (cs33 * rs6);
        J[6] = (-F.dt*(nj6_c3*xt43 + T(3)*tj[J_ch3ccl3])) * (cs34 * rs6);
        J[5] = (-F.dt*(K[K_d95]*xt43 + tj[J_ch3cl])) * (cs35 * rs6);
        J[3] = (-F.dt*(K[K_d96]*xt42 + K[K_d97]*xt43 + tj[J_hcfc22])) * (cs36 * rs6);
        J[1] = (-F.dt*(K[K_e52]*xt42 + tj[J_h1211])) * (cs38 * rs6);
        J[8] = (-F.dt*(T(3)*K[K_d90]*xt30 + T(3)*K[K_d92]*xt32 + K[K_d96]*xt36 + K[K_e52]*xt38 + nj6_c1*xt31 + nj6_c2*xt33)) * (cs42 * rs6);
        J[10] = (-F.dt*(K[K_d95]*xt35 + K[K_d97]*xt36 + nj6_c3*xt34)) * (cs43 * rs6);
    }
    {  // row 8
    const T rs8 = nt_rscale<T>(nt_exp_hi(x[8]), fh);
        const T nj8_c0 = F.dt*K[K_a36];
        J[160] = (nj8_c0*xt43 + T(1)) * (cs8 * rs8);
        J[161] = (-F.dt*tj[J_ch2o_co]) * (cs27 * rs8);
        J[165] = (nj8_c0*xt8) * (cs43 * rs8);
        J[163] = T(0);
        J[162] = T(0);
        J[164] = T(0);
    }
    {  // row 9
    const T rs9 = nt_rscale<T>(nt_exp_hi(x[9]), fh);
        const T nj9_c0 = F.dt*K[K_e5a];
        J[100] = (F.dt*tj[J_oclo] + T(1)) * (cs9 * rs9);
        J[102] = (-nj9_c0*xt53) * (cs52 * rs9);
        J[101] = (-nj9_c0*xt52) * (cs53 * rs9);
    }
    {  // row 10
    const T rs10 = nt_rscale<T>(nt_exp_hi(x[10]), fh);
    }
    {  // row 11
    const T rs11 = nt_rscale<T>(nt_exp_hi(x[11]), fh);
    }
    {  // row 12
    const T rs12 = nt_rscale<T>(nt_exp_hi(x[12]), fh);
        const T nj12_c0 = F.dt*xt44;
        const T nj12_c1 = F.dt*xt12;
        const T nj12_c2 = F.dt*K[K_d9];
        J[250] = (-K[K_d5]*nj12_c0) * (cs1 * rs12);
        J[247] = (het[3]*nj12_c1) * (cs5 * rs12);
        J[253] = (F.dt*(F.parthcl*(K[K_d11]*xt43 + tj[J_hcl]) + F.rain_hcl + het[1]*xt13 + het[3]*xt5 + het[4]*xt14 + het[6]*xt25) + T(1)) * (cs12 * rs12);
        J[249] = (het[1]*nj12_c1) * (cs13 * rs12);
        J[251] = (het[4]*nj12_c1) * (cs14 * rs12);
        J[248] = (het[6]*nj12_c1) * (cs25 * rs12);
        J[252] = (-K[K_c10]*nj12_c0) * (cs27 * rs12);
        J[255] = (F.parthcl*K[K_d11]*nj12_c1 - nj12_c2*xt52) * (cs43 * rs12);
        J[254] = (-F.dt*(F.h2*K[K_d6] + K[K_c10]*xt27 + K[K_d5]*xt1 + K[K_d7]*xt47)) * (cs44 * rs12);
        J[256] = (-K[K_d7]*nj12_c0) * (cs47 * rs12);
        J[257] = (-nj12_c2*xt43) * (cs52 * rs12);
    }
    {  // row 13
    const T rs13 = nt_rscale<T>(nt_exp_hi(x[13]), fh);
        const T nj13_c0 = F.dt*xt13;
        const T nj13_c1 = F.dt*K[K_d31];
        J[89] = (het[0]*nj13_c0) * (cs2 * rs13);
        J[88] = (het[1]*nj13_c0) * (cs12 * rs13);
        J[87] = (F.dt*(K[K_d32]*xt45 + het[0]*xt2 + het[1]*xt12 + tj[J_clono2_cl] + tj[J_clono2_clo]) + T(1)) * (cs13 * rs13);
        J[91] = (K[K_d32]*nj13_c0) * (cs45 * rs13);
        J[90] = (-nj13_c1*xt52) * (cs48 * rs13);
        J[92] = (-nj13_c1*xt48) * (cs52 * rs13);
    }
    {  // row 14
    const T rs14 = nt_rscale<T>(nt_exp_hi(x[14]), fh);
        const T nj14_c0 = F.dt*het[0];
        const T nj14_c1 = F.dt*xt14;
        const T nj14_c2 = F.dt*K[K_d33];
        J[170] = (-nj14_c0*xt13) * (cs2 * rs14);
        J[169] = (het[4]*nj14_c1) * (cs12 * rs14);
        J[166] = (-nj14_c0*xt2) * (cs13 * rs14);
        J[167] = (F.dt*(K[K_d34]*xt43 + K[K_d35]*xt45 + K[K_d37]*xt44 + het[4]*xt12 + het[8]*xt18 + tj[J_hocl]) + T(1)) * (cs14 * rs14);
        J[168] = (het[8]*nj14_c1) * (cs18 * rs14);
        J[173] = (K[K_d34]*nj14_c1) * (cs43 * rs14);
        J[172] = (K[K_d37]*nj14_c1) * (cs44 * rs14);
        J[171] = (K[K_d35]*nj14_c1) * (cs45 * rs14);
        J[174] = (-nj14_c2*xt52) * (cs47 * rs14);
        J[175] = (-nj14_c2*xt47) * (cs52 * rs14);
    }
    {  // row 15
    const T rs15 = nt_rscale<T>(nt_exp_hi(x[15]), fh);
        J[63] = (-F.dt*(het[1]*xt13 + het[4]*xt14)) * (cs12 * rs15);
        J[61] = (-F.dt*het[1]*xt12) * (cs13 * rs15);
        J[62] = (-F.dt*(K[K_d37]*xt44 + het[4]*xt12)) * (cs14 * rs15);
        J[60] = (F.dt*tj[J_cl2] + T(1)) * (cs15 * rs15);
        J[64] = (-F.dt*K[K_d37]*xt14) * (cs44 * rs15);
        J[65] = (-T(2)*F.dt*K[K_d62]*xt52) * (cs52 * rs15);
    }
    {  // row 16
    const T rs16 = nt_rscale<T>(nt_exp_hi(x[16]), fh);
        J[189] = (F.dt*(F.rain_h2o2 + K[K_a30]*xt43 + tj[J_h2o2]) + T(1)) * (cs16 * rs16);
        J[190] = (F.dt*K[K_a30]*xt16) * (cs43 * rs16);
        J[191] = (-T(2)*F.dt*K[K_a27]*xt47) * (cs47 * rs16);
    }
    {  // row 17
    const T rs17 = nt_rscale<T>(nt_exp_hi(x[17]), fh);
        const T nj17_c0 = F.dt*het[3];
        const T nj17_c1 = F.dt*K[K_d36];
        J[26] = (-nj17_c0*xt12) * (cs5 * rs17);
        J[27] = (-nj17_c0*xt5) * (cs12 * rs17);
        J[25] = (F.dt*tj[J_clno2] + T(1)) * (cs17 * rs17);
        J[29] = (-nj17_c1*xt48) * (cs44 * rs17);
        J[28] = (-nj17_c1*xt44) * (cs48 * rs17);
    }
    {  // row 18
    const T rs18 = nt_rscale<T>(nt_exp_hi(x[18]), fh);
        const T nj18_c0 = F.dt*xt18;
        const T nj18_c1 = F.dt*xt50;
        const T nj18_c2 = F.parthbr*nj18_c0;
        J[183] = (het[8]*nj18_c0) * (cs14 * rs18);
        J[184] = (F.dt*(F.parthbr*(K[K_e11]*xt43 + K[K_e9]*xt42 + tj[J_hbr]) + F.rain_hbr + het[7]*xt25 + het[8]*xt14) + T(1)) * (cs18 * rs18);
        J[181] = (het[7]*nj18_c0) * (cs25 * rs18);
        J[185] = (-K[K_c19]*nj18_c1) * (cs27 * rs18);
        J[182] = (K[K_e9]*nj18_c2) * (cs42 * rs18);
        J[187] = (K[K_e11]*nj18_c2) * (cs43 * rs18);
        J[188] = (-K[K_e7]*nj18_c1) * (cs47 * rs18);
        J[186] = (-F.dt*(K[K_c19]*xt27 + K[K_e7]*xt47)) * (cs50 * rs18);
    }
    {  // row 19
    const T rs19 = nt_rscale<T>(nt_exp_hi(x[19]), fh);
        const T nj19_c0 = F.dt*xt19;
        const T nj19_c1 = F.dt*K[K_e13];
        J[56] = (het[5]*nj19_c0) * (cs2 * rs19);
        J[55] = (F.dt*(K[K_e8]*xt45 + het[5]*xt2 + tj[J_brono2]) + T(1)) * (cs19 * rs19);
        J[58] = (K[K_e8]*nj19_c0) * (cs45 * rs19);
        J[57] = (-nj19_c1*xt53) * (cs48 * rs19);
        J[59] = (-nj19_c1*xt48) * (cs53 * rs19);
    }
    {  // row 20
    const T rs20 = nt_rscale<T>(nt_exp_hi(x[20]), fh);
        const T nj20_c0 = T(2)*F.dt;
        const T nj20_c1 = K[K_b39]*nj20_c0;
        const T nj20_c2 = F.parthno3*K[K_b27];
        const T nj20_c3 = F.dt*xt48;
        const T nj20_c4 = T(2)*K[K_b12];
        const T nj20_c5 = K[K_b6]*nj20_c0;
        J[233] = (-nj20_c1*xt42) * (cs0 * rs20);
        J[237] = (-F.dt*(F.parthno3*tj[J_hno3] + nj20_c2*xt43)) * (cs4 * rs20);
        J[232] = (-F.dt*(T(2)*F.hnm*K[K_b32] + T(2)*tj[J_n2o5])) * (cs5 * rs20);
        J[235] = (-F.dt*(K[K_d32]*xt45 + tj[J_clono2_cl] + tj[J_clono2_clo])) * (cs13 * rs20);
        J[229] = (-F.dt*tj[J_clno2]) * (cs17 * rs20);
        J[230] = (-F.dt*(K[K_e8]*xt45 + tj[J_brono2])) * (cs19 * rs20);
        J[238] = (-F.dt*(F.hnm*K[K_b24] + K[K_b28]*xt43 + tj[J_hno4])) * (cs21 * rs20);
        J[236] = (-nj20_c1*xt0) * (cs42 * rs20);
        J[243] = (-F.dt*(K[K_b28]*xt21 + nj20_c2*xt4) + K[K_b22]*nj20_c3) * (cs43 * rs20);
        J[241] = (K[K_d36]*nj20_c3) * (cs44 * rs20);
        J[240] = (-F.dt*(K[K_d32]*xt13 + K[K_e8]*xt19)) * (cs45 * rs20);
        J[244] = (K[K_b23]*nj20_c3) * (cs47 * rs20);
        J[239] = (F.dt*(K[K_b22]*xt43 + K[K_b23]*xt47 + K[K_d31]*xt52 + K[K_d36]*xt44 + K[K_e13]*xt53 + nj20_c4*xt54)) * (cs48 * rs20);
        J[245] = (nj20_c5*xt51) * (cs49 * rs20);
        J[234] = (nj20_c5*xt49) * (cs51 * rs20);
        J[246] = (K[K_d31]*nj20_c3) * (cs52 * rs20);
        J[242] = (K[K_e13]*nj20_c3) * (cs53 * rs20);
        J[231] = (nj20_c3*nj20_c4) * (cs54 * rs20);
    }
    {  // row 21
    const T rs21 = nt_rscale<T>(nt_exp_hi(x[21]), fh);
        const T nj21_c0 = F.dt*K[K_b23];
        J[152] = (F.dt*(F.hnm*K[K_b24] + K[K_b28]*xt43 + tj[J_hno4]) + T(1)) * (cs21 * rs21);
        J[154] = (F.dt*K[K_b28]*xt21) * (cs43 * rs21);
        J[155] = (-nj21_c0*xt48) * (cs47 * rs21);
        J[153] = (-nj21_c0*xt47) * (cs48 * rs21);
    }
    {  // row 22
    const T rs22 = nt_rscale<T>(nt_exp_hi(x[22]), fh);
        const T nj22_c0 = F.dt*xt44;
        const T nj22_c1 = T(3)*xt42;
        const T nj22_c2 = T(2)*K[K_d91];
        const T nj22_c3 = T(4)*K[K_d93];
        const T nj22_c4 = T(3)*K[K_d94];
        const T nj22_c5 = F.dt*xt52;
        const T nj22_c6 = T(2)*K[K_d60];
        const T nj22_c7 = T(2)*K[K_d62];
        J[141] = (K[K_d5]*nj22_c0) * (cs1 * rs22);
        J[140] = (-F.dt*tj[J_oclo]) * (cs9 * rs22);
        J[144] = (-F.dt*F.parthcl*(K[K_d11]*xt43 + tj[J_hcl])) * (cs12 * rs22);
        J[135] = (-F.dt*(K[K_d32]*xt45 + tj[J_clono2_cl] + tj[J_clono2_clo])) * (cs13 * rs22);
        J[142] = (-F.dt*(K[K_d34]*xt43 + K[K_d35]*xt45 + tj[J_hocl]) + K[K_d37]*nj22_c0) * (cs14 * rs22);
        J[133] = (-T(2)*F.dt*tj[J_cl2]) * (cs15 * rs22);
        J[128] = (-F.dt*tj[J_clno2]) * (cs17 * rs22);
        J[138] = (-F.dt*(T(2)*F.hnm*K[K_d61] + T(2)*tj[J_cl2o2])) * (cs24 * rs22);
        J[132] = (-F.dt*tj[J_brcl]) * (cs26 * rs22);
        J[143] = (K[K_c10]*nj22_c0) * (cs27 * rs22);
        J[137] = (-F.dt*(K[K_d90]*nj22_c1 + T(3)*tj[J_cfc11])) * (cs30 * rs22);
        J[131] = (-F.dt*(nj22_c2*xt42 + T(2)*tj[J_cfc12])) * (cs31 * rs22);
        J[127] = (-F.dt*(K[K_d92]*nj22_c1 + T(3)*tj[J_cfc113])) * (cs32 * rs22);
        J[129] = (-F.dt*(nj22_c3*xt42 + T(4)*tj[J_ccl4])) * (cs33 * rs22);
        J[136] = (-F.dt*(nj22_c4*xt43 + T(3)*tj[J_ch3ccl3])) * (cs34 * rs22);
        J[134] = (-F.dt*(K[K_d95]*xt43 + tj[J_ch3cl])) * (cs35 * rs22);
        J[130] = (-F.dt*(K[K_d96]*xt42 + K[K_d97]*xt43 + tj[J_hcfc22])) * (cs36 * rs22);
        J[139] = (-F.dt*(T(3)*K[K_d90]*xt30 + T(3)*K[K_d92]*xt32 + K[K_d96]*xt36 + nj22_c2*xt31 + nj22_c3*xt33)) * (cs42 * rs22);
        J[149] = (-F.dt*(F.parthcl*K[K_d11]*xt12 + K[K_d34]*xt14 + K[K_d95]*xt35 + K[K_d97]*xt36 + nj22_c4*xt34) + K[K_d9]*nj22_c5) * (cs43 * rs22);
        J[147] = (F.dt*(F.h2*K[K_d6] + K[K_c10]*xt27 + K[K_d36]*xt48 + K[K_d37]*xt14 + K[K_d5]*xt1 + K[K_d7]*xt47)) * (cs44 * rs22);
        J[146] = (-F.dt*(K[K_d32]*xt13 + K[K_d35]*xt14)) * (cs45 * rs22);
        J[150] = (F.dt*(K[K_d33]*xt52 + K[K_d7]*xt44)) * (cs47 * rs22);
        J[145] = (F.dt*(K[K_d31]*xt52 + K[K_d36]*xt44)) * (cs48 * rs22);
        J[151] = (F.dt*(K[K_d31]*xt48 + K[K_d33]*xt47 + K[K_d9]*xt43 + K[K_e5a]*xt53 + K[K_e5c]*xt53 + nj22_c6*xt52 + nj22_c7*xt52 + xt52*(nj22_c6 + nj22_c7))) * (cs52 * rs22);
        J[148] = (nj22_c5*(K[K_e5a] + K[K_e5c])) * (cs53 * rs22);
    }
    {  // row 23
    const T rs23 = nt_rscale<T>(nt_exp_hi(x[23]), fh);
        const T nj23_c0 = T(2)*het[7];
        const T nj23_c1 = F.dt*F.parthbr*xt18;
        const T nj23_c2 = F.dt*xt53;
        J[196] = (-F.dt*(F.parthbr*(K[K_e11]*xt43 + K[K_e9]*xt42 + tj[J_hbr]) + nj23_c0*xt25)) * (cs18 * rs23);
        J[193] = (-F.dt*(K[K_e8]*xt45 + tj[J_brono2])) * (cs19 * rs23);
        J[194] = (-F.dt*(K[K_e16]*xt45 + nj23_c0*xt18 + tj[J_hobr])) * (cs25 * rs23);
        J[192] = (-F.dt*tj[J_brcl]) * (cs26 * rs23);
        J[197] = (F.dt*K[K_c19]*xt50) * (cs27 * rs23);
        J[195] = (-K[K_e9]*nj23_c1) * (cs42 * rs23);
        J[202] = (-K[K_e11]*nj23_c1) * (cs43 * rs23);
        J[199] = (-F.dt*(K[K_e16]*xt25 + K[K_e8]*xt19)) * (cs45 * rs23);
        J[203] = (F.dt*(K[K_e15]*xt53 + K[K_e7]*xt50)) * (cs47 * rs23);
        J[198] = (K[K_e13]*nj23_c2) * (cs48 * rs23);
        J[201] = (F.dt*(K[K_c19]*xt27 + K[K_e7]*xt47)) * (cs50 * rs23);
        J[204] = (K[K_e5c]*nj23_c2) * (cs52 * rs23);
        J[200] = (F.dt*(K[K_e13]*xt48 + K[K_e15]*xt47 + K[K_e5c]*xt52)) * (cs53 * rs23);
    }
    {  // row 24
    const T rs24 = nt_rscale<T>(nt_exp_hi(x[24]), fh);
        J[97] = (F.dt*(F.hnm*K[K_d61] + tj[J_cl2o2]) + T(1)) * (cs24 * rs24);
        J[98] = (-T(2)*F.dt*K[K_d60]*xt52) * (cs52 * rs24);
    }
    {  // row 25
    const T rs25 = nt_rscale<T>(nt_exp_hi(x[25]), fh);
        const T nj25_c0 = F.dt*het[5];
        const T nj25_c1 = F.dt*xt25;
        const T nj25_c2 = F.dt*K[K_e15];
        J[83] = (-nj25_c0*xt19) * (cs2 * rs25);
        J[82] = (het[6]*nj25_c1) * (cs12 * rs25);
        J[81] = (het[7]*nj25_c1) * (cs18 * rs25);
        J[79] = (-nj25_c0*xt2) * (cs19 * rs25);
        J[80] = (F.dt*(K[K_e16]*xt45 + het[6]*xt12 + het[7]*xt18 + tj[J_hobr]) + T(1)) * (cs25 * rs25);
        J[84] = (K[K_e16]*nj25_c1) * (cs45 * rs25);
        J[86] = (-nj25_c2*xt53) * (cs47 * rs25);
        J[85] = (-nj25_c2*xt47) * (cs53 * rs25);
    }
    {  // row 26
    const T rs26 = nt_rscale<T>(nt_exp_hi(x[26]), fh);
        const T nj26_c0 = F.dt*het[6];
        const T nj26_c1 = F.dt*het[8];
        const T nj26_c2 = F.dt*K[K_e5c];
        J[47] = (-nj26_c0*xt25) * (cs12 * rs26);
        J[45] = (-nj26_c1*xt18) * (cs14 * rs26);
        J[46] = (-nj26_c1*xt14) * (cs18 * rs26);
        J[44] = (-nj26_c0*xt12) * (cs25 * rs26);
        J[43] = (F.dt*tj[J_brcl] + T(1)) * (cs26 * rs26);
        J[49] = (-nj26_c2*xt53) * (cs52 * rs26);
        J[48] = (-nj26_c2*xt52) * (cs53 * rs26);
    }
    {  // row 27
    const T rs27 = nt_rscale<T>(nt_exp_hi(x[27]), fh);
        const T nj27_c0 = F.dt*K[K_c1c];
        const T nj27_c1 = F.dt*K[K_c17b];
        const T nj27_c2 = F.dt*xt27;
        const T nj27_c3 = F.dt*K[K_c3];
        J[219] = (-nj27_c0*xt42) * (cs1 * rs27);
        J[222] = (F.dt*(K[K_c10]*xt44 + K[K_c19]*xt50 + K[K_c8]*xt43 + K[K_c9]*xt45 + tj[J_ch2o_co] + tj[J_ch2o_hco]) + T(1)) * (cs27 * rs27);
        J[221] = T(0);
        J[217] = (-nj27_c1*xt43) * (cs29 * rs27);
        J[218] = (-nj27_c0*xt1) * (cs42 * rs27);
        J[226] = (F.dt*K[K_c8]*xt27 - nj27_c1*xt29) * (cs43 * rs27);
        J[224] = (K[K_c10]*nj27_c2) * (cs44 * rs27);
        J[223] = (F.dt*K[K_c9]*xt27 - nj27_c3*xt56) * (cs45 * rs27);
        J[227] = T(0);
        J[225] = (K[K_c19]*nj27_c2) * (cs50 * rs27);
        J[228] = T(0);
        J[220] = (-nj27_c3*xt45) * (cs56 * rs27);
    }
    {  // row 28
    const T rs28 = nt_rscale<T>(nt_exp_hi(x[28]), fh);
        const T nj28_c0 = T(2)*K[K_c14]*xt28;
        const T nj28_c1 = F.dt*K[K_c17a];
        const T nj28_c2 = F.dt*xt28;
        J[212] = (F.dt*nj28_c0 + F.dt*(K[K_c18]*xt52 + K[K_c5]*xt49 + K[K_c7]*xt47 + nj28_c0) + T(1)) * (cs28 * rs28);
        J[210] = (-nj28_c1*xt43) * (cs29 * rs28);
        J[213] = (-nj28_c1*xt29) * (cs43 * rs28);
        J[214] = (K[K_c7]*nj28_c2) * (cs47 * rs28);
        J[215] = (K[K_c5]*nj28_c2) * (cs49 * rs28);
        J[216] = (K[K_c18]*nj28_c2) * (cs52 * rs28);
        J[211] = (-F.dt*F.o2*K[K_c4]) * (cs56 * rs28);
    }
    {  // row 29
    const T rs29 = nt_rscale<T>(nt_exp_hi(x[29]), fh);
        const T nj29_c0 = F.dt*K[K_c7];
        J[35] = (-nj29_c0*xt47) * (cs28 * rs29);
        J[34] = (F.dt*(K[K_c17a]*xt43 + K[K_c17b]*xt43 + tj[J_ch3o2h]) + T(1)) * (cs29 * rs29);
        J[36] = (F.dt*xt29*(K[K_c17a] + K[K_c17b])) * (cs43 * rs29);
        J[37] = (-nj29_c0*xt28) * (cs47 * rs29);
    }
    {  // row 30
    const T rs30 = nt_rscale<T>(nt_exp_hi(x[30]), fh);
        J[95] = (F.dt*(K[K_d90]*xt42 + tj[J_cfc11]) + T(1)) * (cs30 * rs30);
        J[96] = (F.dt*K[K_d90]*xt30) * (cs42 * rs30);
    }
    {  // row 31
    const T rs31 = nt_rscale<T>(nt_exp_hi(x[31]), fh);
        J[41] = (F.dt*(K[K_d91]*xt42 + tj[J_cfc12]) + T(1)) * (cs31 * rs31);
        J[42] = (F.dt*K[K_d91]*xt31) * (cs42 * rs31);
    }
    {  // row 32
    const T rs32 = nt_rscale<T>(nt_exp_hi(x[32]), fh);
        J[18] = (F.dt*(K[K_d92]*xt42 + tj[J_cfc113]) + T(1)) * (cs32 * rs32);
        J[19] = (F.dt*K[K_d92]*xt32) * (cs42 * rs32);
    }
    {  // row 33
    const T rs33 = nt_rscale<T>(nt_exp_hi(x[33]), fh);
        J[32] = (F.dt*(K[K_d93]*xt42 + tj[J_ccl4]) + T(1)) * (cs33 * rs33);
        J[33] = (F.dt*K[K_d93]*xt33) * (cs42 * rs33);
    }
    {  // row 34
    const T rs34 = nt_rscale<T>(nt_exp_hi(x[34]), fh);
        J[93] = (F.dt*(K[K_d94]*xt43 + tj[J_ch3ccl3]) + T(1)) * (cs34 * rs34);
        J[94] = (F.dt*K[K_d94]*xt34) * (cs43 * rs34);
    }
    {  // row 35
    const T rs35 = nt_rscale<T>(nt_exp_hi(x[35]), fh);
        J[66] = (F.dt*(K[K_d95]*xt43 + tj[J_ch3cl]) + T(1)) * (cs35 * rs35);
        J[67] = (F.dt*K[K_d95]*xt35) * (cs43 * rs35);
    }
    {  // row 36
    const T rs36 = nt_rscale<T>(nt_exp_hi(x[36]), fh);
        const T nj36_c0 = F.dt*xt36;
        J[38] = (F.dt*(K[K_d96]*xt42 + K[K_d97]*xt43 + tj[J_hcfc22]) + T(1)) * (cs36 * rs36);
        J[39] = (K[K_d96]*nj36_c0) * (cs42 * rs36);
        J[40] = (K[K_d97]*nj36_c0) * (cs43 * rs36);
    }
    {  // row 37
    const T rs37 = nt_rscale<T>(nt_exp_hi(x[37]), fh);
        const T nj37_c0 = F.dt*xt37;
        J[52] = (F.dt*(K[K_e50]*xt42 + K[K_e51]*xt43 + tj[J_ch3br]) + T(1)) * (cs37 * rs37);
        J[53] = (K[K_e50]*nj37_c0) * (cs42 * rs37);
        J[54] = (K[K_e51]*nj37_c0) * (cs43 * rs37);
    }
    {  // row 38
    const T rs38 = nt_rscale<T>(nt_exp_hi(x[38]), fh);
        J[30] = (F.dt*(K[K_e52]*xt42 + tj[J_h1211]) + T(1)) * (cs38 * rs38);
        J[31] = (F.dt*K[K_e52]*xt38) * (cs42 * rs38);
    }
    {  // row 39
    const T rs39 = nt_rscale<T>(nt_exp_hi(x[39]), fh);
        J[50] = (F.dt*(K[K_e53]*xt42 + tj[J_h1301]) + T(1)) * (cs39 * rs39);
        J[51] = (F.dt*K[K_e53]*xt39) * (cs42 * rs39);
    }
    {  // row 40
    const T rs40 = nt_rscale<T>(nt_exp_hi(x[40]), fh);
        const T nj40_c0 = T(2)*K[K_e54];
        J[16] = (F.dt*F.rain_hbr) * (cs18 * rs40);
        J[13] = (-F.dt*(K[K_e50]*xt42 + K[K_e51]*xt43 + tj[J_ch3br])) * (cs37 * rs40);
        J[11] = (-F.dt*(K[K_e52]*xt42 + tj[J_h1211])) * (cs38 * rs40);
        J[12] = (-F.dt*(K[K_e53]*xt42 + tj[J_h1301])) * (cs39 * rs40);
        J[15] = (-F.dt*(nj40_c0*xt43 + T(2)*tj[J_ch2br2])) * (cs41 * rs40);
        J[14] = (-F.dt*(K[K_e50]*xt37 + K[K_e52]*xt38 + K[K_e53]*xt39)) * (cs42 * rs40);
        J[17] = (-F.dt*(K[K_e51]*xt37 + nj40_c0*xt41)) * (cs43 * rs40);
    }
    {  // row 41
    const T rs41 = nt_rscale<T>(nt_exp_hi(x[41]), fh);
        J[125] = (F.dt*(K[K_e54]*xt43 + tj[J_ch2br2]) + T(1)) * (cs41 * rs41);
        J[126] = (F.dt*K[K_e54]*xt41) * (cs43 * rs41);
    }
    {  // row 42
    const T rs42 = nt_rscale<T>(nt_exp_hi(x[42]), fh);
        J[99] = T(0);
    }
    {  // row 43
    const T rs43 = nt_rscale<T>(nt_exp_hi(x[43]), fh);
        J[321] = T(0);
        J[331] = T(0);
        J[319] = T(0);
        J[322] = T(0);
        J[330] = T(0);
        J[323] = T(0);
        J[326] = T(0);
        J[325] = T(0);
        J[320] = T(0);
        J[317] = T(0);
        J[329] = T(0);
        J[328] = T(0);
        J[316] = T(0);
        J[318] = T(0);
        J[337] = (T(1)) * (cs43 * rs43);
        J[334] = T(0);
        J[333] = T(0);
        J[339] = T(0);
        J[338] = T(0);
        J[332] = T(0);
        J[340] = T(0);
        J[336] = T(0);
        J[341] = T(0);
        J[335] = T(0);
        J[327] = T(0);
        J[324] = T(0);
    }
    {  // row 44
    const T rs44 = nt_rscale<T>(nt_exp_hi(x[44]), fh);
        J[284] = T(0);
        J[288] = T(0);
        J[287] = T(0);
        J[285] = T(0);
        J[286] = T(0);
        J[292] = T(0);
        J[290] = T(0);
        J[294] = T(0);
        J[293] = T(0);
        J[289] = T(0);
        J[295] = T(0);
        J[296] = T(0);
        J[291] = T(0);
    }
    {  // row 45
    const T rs45 = nt_rscale<T>(nt_exp_hi(x[45]), fh);
        J[280] = T(0);
        J[279] = T(0);
        J[282] = T(0);
        J[281] = T(0);
        J[283] = T(0);
        J[278] = T(0);
    }
    {  // row 46
    const T rs46 = nt_rscale<T>(nt_exp_hi(x[46]), fh);
        J[355] = (T(-1)) * (cs7 * rs46);
        J[358] = T(0);
        J[357] = T(0);
        J[359] = T(0);
        J[360] = T(0);
        J[356] = T(0);
    }
    {  // row 47
    const T rs47 = nt_rscale<T>(nt_exp_hi(x[47]), fh);
        J[342] = T(0);
        J[343] = T(0);
        J[345] = T(0);
        J[350] = T(0);
        J[347] = T(0);
        J[346] = T(0);
        J[352] = T(0);
        J[351] = (T(1)) * (cs47 * rs47);
        J[353] = T(0);
        J[349] = T(0);
        J[354] = T(0);
        J[348] = T(0);
        J[344] = T(0);
    }
    {  // row 49
    const T rs49 = nt_rscale<T>(nt_exp_hi(x[49]), fh);
        J[361] = T(0);
        J[363] = T(0);
        J[366] = T(0);
        J[365] = T(0);
        J[362] = T(0);
        J[367] = T(0);
        J[364] = T(0);
    }
    {  // row 50
    const T rs50 = nt_rscale<T>(nt_exp_hi(x[50]), fh);
        J[307] = T(0);
        J[311] = T(0);
        J[309] = T(0);
        J[313] = T(0);
        J[312] = T(0);
        J[308] = T(0);
        J[314] = T(0);
        J[315] = T(0);
        J[310] = T(0);
    }
    {  // row 51
    const T rs51 = nt_rscale<T>(nt_exp_hi(x[51]), fh);
        J[78] = T(0);
    }
    {  // row 55
    const T rs55 = nt_rscale<T>(nt_exp_hi(x[55]), fh);
        J[205] = T(0);
        J[207] = T(0);
        J[206] = T(0);
        J[209] = T(0);
        J[208] = T(0);
    }
    {  // row 56
    const T rs56 = nt_rscale<T>(nt_exp_hi(x[56]), fh);
        J[177] = T(0);
        J[176] = T(0);
        J[180] = T(0);
        J[179] = T(0);
        J[178] = T(0);
    }
    const T N_cno_c0 = nt_div<T>(K[K_b9], K[K_b12]);
    const T N_cno = N_cno_c0*xt46;
    const T d_N_cno_46 = N_cno_c0;
    const T N_dno = -N_cno + xt20;
    const T d_N_dno_20 = T(1);
    const T d_N_dno_46 = -d_N_cno_46;
    const T N_no2_c0 = N_cno + T(1e-30);
    const T N_no2_c1 = nt_div<T>(T(1e-30), N_no2_c0);
    const bool sel_N_no2 = (N_dno) > (T(1e-30));
    const T N_no2 = sel_N_no2 ? T(N_dno) : T(N_no2_c1*xt20);
    const T d_N_no2_20 = sel_N_no2 ? T(d_N_dno_20) : T(N_no2_c1);
    const T d_N_no2_46 = sel_N_no2 ? T(d_N_dno_46) : T(nt_div<T>(-T(1e-30)*d_N_cno_46*xt20, (N_no2_c0*N_no2_c0)));
    {  // row 48
    const T rs48 = nt_rscale<T>(nt_exp_hi(x[48]), fh);
        J[270] = (-d_N_no2_20) * (cs20 * rs48);
        J[269] = T(0);
        J[272] = T(0);
        J[275] = (-d_N_no2_46) * (cs46 * rs48);
        J[274] = T(0);
        J[271] = (T(1)) * (cs48 * rs48);
        J[276] = T(0);
        J[277] = T(0);
        J[273] = T(0);
    }
    const T N_no3_c0 = N_cno + T(1e-30);
    const T N_no3_c1 = nt_div<T>(T(1), N_no3_c0);
    const T N_no3_c2 = N_cno*N_no3_c1;
    const bool sel_N_no3 = (N_dno) > (T(1e-30));
    const T N_no3 = sel_N_no3 ? T(N_cno) : T(N_no3_c2*xt20);
    const T d_N_no3_20 = sel_N_no3 ? T(T(0)) : T(N_no3_c2);
    const T d_N_no3_46 = sel_N_no3 ? T(d_N_cno_46) : T(d_N_cno_46*(nt_div<T>(-N_cno*xt20, (N_no3_c0*N_no3_c0)) + N_no3_c1*xt20));
    {  // row 54
    const T rs54 = nt_rscale<T>(nt_exp_hi(x[54]), fh);
        J[68] = (-d_N_no3_20) * (cs20 * rs54);
        J[70] = (-d_N_no3_46) * (cs46 * rs54);
        J[69] = T(0);
    }
    const bool sel_N_clo = (xt22) >= (T(0));
    const T N_clo = sel_N_clo ? T(xt22) : T(T(0));
    const T d_N_clo_22 = sel_N_clo ? T(T(1)) : T(T(0));
    {  // row 52
    const T rs52 = nt_rscale<T>(nt_exp_hi(x[52]), fh);
        J[369] = T(0);
        J[373] = T(0);
        J[372] = T(0);
        J[370] = T(0);
        J[368] = (-d_N_clo_22) * (cs22 * rs52);
        J[371] = T(0);
        J[377] = T(0);
        J[375] = T(0);
        J[379] = T(0);
        J[378] = T(0);
        J[374] = T(0);
        J[380] = T(0);
        J[381] = (T(1)) * (cs52 * rs52);
        J[376] = T(0);
    }
    const bool sel_N_bro = (xt23) >= (T(0));
    const T N_bro = sel_N_bro ? T(xt23) : T(T(0));
    const T d_N_bro_23 = sel_N_bro ? T(T(1)) : T(T(0));
    {  // row 53
    const T rs53 = nt_rscale<T>(nt_exp_hi(x[53]), fh);
        J[297] = (-d_N_bro_23) * (cs23 * rs53);
        J[298] = T(0);
        J[302] = T(0);
        J[300] = T(0);
        J[304] = T(0);
        J[303] = T(0);
        J[299] = T(0);
        J[305] = T(0);
        J[306] = T(0);
        J[301] = (T(1)) * (cs53 * rs53);
    }
    const T N_t06_c0 = tj[J_hocl]*xt14;
    const T N_t06_c1 = K[K_d33]*xt52;
    const T N_t06_c2 = N_t06_c1*xt47;
    const bool sel_N_t06 = (N_t06_c0) <= (N_t06_c2);
    const T N_t06 = sel_N_t06 ? T(N_t06_c0) : T(N_t06_c2);
    const T d_N_t06_14 = sel_N_t06 ? T(tj[J_hocl]) : T(T(0));
    const T d_N_t06_47 = sel_N_t06 ? T(T(0)) : T(N_t06_c1);
    const T d_N_t06_52 = sel_N_t06 ? T(T(0)) : T(K[K_d33]*xt47);
    const T N_t07_c0 = K[K_e5c]*xt53;
    const T N_t07_c1 = N_t07_c0*xt52;
    const T N_t07_c2 = tj[J_brcl]*xt26;
    const bool sel_N_t07 = (N_t07_c1) <= (N_t07_c2);
    const T N_t07 = sel_N_t07 ? T(N_t07_c1) : T(N_t07_c2);
    const T d_N_t07_26 = sel_N_t07 ? T(T(0)) : T(tj[J_brcl]);
    const T d_N_t07_52 = sel_N_t07 ? T(N_t07_c0) : T(T(0));
    const T d_N_t07_53 = sel_N_t07 ? T(K[K_e5c]*xt52) : T(T(0));
    const T N_t09_c0 = K[K_e15]*xt53;
    const T N_t09_c1 = N_t09_c0*xt47;
    const T N_t09_c2 = tj[J_hobr]*xt25;
    const bool sel_N_t09 = (N_t09_c1) <= (N_t09_c2);
    const T N_t09 = sel_N_t09 ? T(N_t09_c1) : T(N_t09_c2);
    const T d_N_t09_25 = sel_N_t09 ? T(T(0)) : T(tj[J_hobr]);
    const T d_N_t09_47 = sel_N_t09 ? T(N_t09_c0) : T(T(0));
    const T d_N_t09_53 = sel_N_t09 ? T(K[K_e15]*xt47) : T(T(0));
    {  // row 7
    const T rs7 = nt_rscale<T>(nt_exp_hi(x[7]), fh);
        const T nj7_c0 = T(2)*F.dt;
        const T nj7_c1 = nt_div<T>(tj[J_no3_no], fmax(T(1e-30), tj[J_no3_no2] + tj[J_no3_no]));
        const T nj7_c2 = F.dt*xt49;
        const T nj7_c3 = T(2)*K[K_b3];
        const T nj7_c4 = T(2)*K[K_d3];
        const T nj7_c5 = T(2)*K[K_hk3];
        const T nj7_c6 = T(2)*K[K_b9]*nj7_c1;
        J[105] = (nj7_c0*nj7_c1*tj[J_clono2_cl]) * (cs13 * rs7);
        J[106] = (F.dt*d_N_t06_14) * (cs14 * rs7);
        J[104] = (F.dt*d_N_t09_25) * (cs25 * rs7);
        J[103] = (d_N_t07_26*nj7_c0) * (cs26 * rs7);
        J[108] = (-K[K_c5]*nj7_c2) * (cs28 * rs7);
        J[112] = (F.dt*(K[K_a5]*xt45 + K[K_a6]*xt46)) * (cs43 * rs7);
        J[110] = (F.dt*(K[K_a5]*xt43 + K[K_a7]*xt47 + T(4)*K[K_hk1]*xt45 + nj7_c3*xt48 + nj7_c4*xt52 + nj7_c5*xt46)) * (cs45 * rs7);
        J[114] = (F.dt*(K[K_a2]*xt55 + K[K_a6]*xt43 + K[K_a6b]*xt47 + nj7_c5*xt45 + nj7_c6*xt48)) * (cs46 * rs7);
        J[113] = (F.dt*d_N_t06_47 + F.dt*d_N_t09_47 + F.dt*(K[K_a6b]*xt46 + K[K_a7]*xt45) - K[K_a26]*nj7_c2) * (cs47 * rs7);
        J[109] = (F.dt*(nj7_c3*xt45 + nj7_c6*xt46)) * (cs48 * rs7);
        J[115] = (-F.dt*(K[K_a26]*xt47 + K[K_c5]*xt28)) * (cs49 * rs7);
        J[116] = (F.dt*d_N_t06_52 + F.dt*(nt_div<T>(T(4)*K[K_d60]*tj[J_cl2o2]*xt52, F.hnm*K[K_d61] + tj[J_cl2o2]) + nj7_c4*xt45) + d_N_t07_52*nj7_c0) * (cs52 * rs7);
        J[111] = (F.dt*d_N_t09_53 + d_N_t07_53*nj7_c0) * (cs53 * rs7);
        J[107] = (F.dt*K[K_a2]*xt46) * (cs55 * rs7);
    }
}

// residual rows [3, 4, 6, 8, 11, 13, 15, 16, 18, 21, 22, 23, 26, 27, 30, 32, 34, 37, 38, 41, 42, 43, 45, 48, 49, 51, 53, 54, 56] (night equations, FP64)
template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>
__device__ __forceinline__ void nt_residual_night_w2_0(const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {
    R[3] = -T(2)*F.dt*K[K_b39]*x[0]*x[42] + F.dt*(F.rain_hno3*x[4] + T(2)*K[K_b6]*x[49]*x[51]) - ck0[3] + x[3];
    R[4] = -F.dt*(K[K_b22]*x[43]*x[48] + het[0]*x[13]*x[2] + het[1]*x[12]*x[13] + T(2)*het[2]*x[2]*x[5] + het[3]*x[12]*x[5] + het[5]*x[19]*x[2]) - ck0[4] + x[4]*(F.dt*(F.parthno3*(K[K_b27]*x[43] + tj[J_hno3]) + F.rain_hno3) + T(1));
    const T nr6_c0 = T(3)*x[42];
    R[6] = F.dt*F.rain_hcl*x[12] - F.dt*(x[30]*(K[K_d90]*nr6_c0 + T(3)*tj[J_cfc11]) + x[31]*(T(2)*K[K_d91]*x[42] + T(2)*tj[J_cfc12]) + x[32]*(K[K_d92]*nr6_c0 + T(3)*tj[J_cfc113]) + x[33]*(T(4)*K[K_d93]*x[42] + T(4)*tj[J_ccl4]) + x[34]*(T(3)*K[K_d94]*x[43] + T(3)*tj[J_ch3ccl3]) + x[35]*(K[K_d95]*x[43] + tj[J_ch3cl]) + x[36]*(K[K_d96]*x[42] + K[K_d97]*x[43] + tj[J_hcfc22]) + x[38]*(K[K_e52]*x[42] + tj[J_h1211])) - ck0[6] + x[6];
    R[8] = -F.dt*(F.co2*tj[J_co2] + tj[J_ch2o_co]*x[27]) - ck0[8] + x[8]*(F.dt*K[K_a36]*x[43] + T(1));
    R[11] = -ck0[11] + x[11];
    R[13] = -F.dt*K[K_d31]*x[48]*x[52] - ck0[13] + x[13]*(F.dt*(K[K_d32]*x[45] + het[0]*x[2] + het[1]*x[12] + tj[J_clono2_cl] + tj[J_clono2_clo]) + T(1));
    R[15] = -F.dt*(K[K_d37]*x[14]*x[44] + K[K_d62]*(x[52]*x[52]) + het[1]*x[12]*x[13] + het[4]*x[12]*x[14]) - ck0[15] + x[15]*(F.dt*tj[J_cl2] + T(1));
    R[16] = -F.dt*K[K_a27]*(x[47]*x[47]) - ck0[16] + x[16]*(F.dt*(F.rain_h2o2 + K[K_a30]*x[43] + tj[J_h2o2]) + T(1));
    R[18] = -F.dt*(K[K_c19]*x[27]*x[50] + K[K_e7]*x[47]*x[50]) - ck0[18] + x[18]*(F.dt*(F.parthbr*(K[K_e11]*x[43] + K[K_e9]*x[42] + tj[J_hbr]) + F.rain_hbr + het[7]*x[25] + het[8]*x[14]) + T(1));
    R[21] = -F.dt*K[K_b23]*x[47]*x[48] - ck0[21] + x[21]*(F.dt*(F.hnm*K[K_b24] + K[K_b28]*x[43] + tj[J_hno4]) + T(1));
    const T nr22_c0 = T(2)*x[52];
    const T nr22_c1 = T(3)*x[42];
    R[22] = F.dt*(x[44]*(F.h2*K[K_d6] + K[K_c10]*x[27] + K[K_d36]*x[48] + K[K_d37]*x[14] + K[K_d5]*x[1] + K[K_d7]*x[47]) + x[52]*(K[K_d31]*x[48] + K[K_d33]*x[47] + K[K_d60]*nr22_c0 + K[K_d62]*nr22_c0 + K[K_d9]*x[43] + K[K_e5a]*x[53] + K[K_e5c]*x[53])) - F.dt*(F.parthcl*x[12]*(K[K_d11]*x[43] + tj[J_hcl]) + tj[J_brcl]*x[26] + T(2)*tj[J_cl2]*x[15] + tj[J_clno2]*x[17] + tj[J_oclo]*x[9] + x[13]*(K[K_d32]*x[45] + tj[J_clono2_cl] + tj[J_clono2_clo]) + x[14]*(K[K_d34]*x[43] + K[K_d35]*x[45] + tj[J_hocl]) + x[24]*(T(2)*F.hnm*K[K_d61] + T(2)*tj[J_cl2o2]) + x[30]*(K[K_d90]*nr22_c1 + T(3)*tj[J_cfc11]) + x[31]*(T(2)*K[K_d91]*x[42] + T(2)*tj[J_cfc12]) + x[32]*(K[K_d92]*nr22_c1 + T(3)*tj[J_cfc113]) + x[33]*(T(4)*K[K_d93]*x[42] + T(4)*tj[J_ccl4]) + x[34]*(T(3)*K[K_d94]*x[43] + T(3)*tj[J_ch3ccl3]) + x[35]*(K[K_d95]*x[43] + tj[J_ch3cl]) + x[36]*(K[K_d96]*x[42] + K[K_d97]*x[43] + tj[J_hcfc22])) - ck0[22] + x[22];
    R[23] = F.dt*(K[K_c19]*x[27]*x[50] + K[K_e7]*x[47]*x[50] + x[53]*(K[K_e13]*x[48] + K[K_e15]*x[47] + K[K_e5c]*x[52])) - F.dt*(F.parthbr*x[18]*(K[K_e11]*x[43] + K[K_e9]*x[42] + tj[J_hbr]) + K[K_e16]*x[25]*x[45] + K[K_e8]*x[19]*x[45] + T(2)*het[7]*x[18]*x[25] + tj[J_brcl]*x[26] + tj[J_brono2]*x[19] + tj[J_hobr]*x[25]) - ck0[23] + x[23];
    R[26] = -F.dt*(K[K_e5c]*x[52]*x[53] + het[6]*x[12]*x[25] + het[8]*x[14]*x[18]) - ck0[26] + x[26]*(F.dt*tj[J_brcl] + T(1));
    R[27] = -F.dt*(K[K_c17b]*x[29]*x[43] + K[K_c1c]*x[1]*x[42] + K[K_c3]*x[45]*x[56]) - ck0[27] + x[27]*(F.dt*(K[K_c10]*x[44] + K[K_c19]*x[50] + K[K_c8]*x[43] + K[K_c9]*x[45] + tj[J_ch2o_co] + tj[J_ch2o_hco]) + T(1));
    R[30] = -ck0[30] + x[30]*(F.dt*(K[K_d90]*x[42] + tj[J_cfc11]) + T(1));
    R[32] = -ck0[32] + x[32]*(F.dt*(K[K_d92]*x[42] + tj[J_cfc113]) + T(1));
    R[34] = -ck0[34] + x[34]*(F.dt*(K[K_d94]*x[43] + tj[J_ch3ccl3]) + T(1));
    R[37] = -ck0[37] + x[37]*(F.dt*(K[K_e50]*x[42] + K[K_e51]*x[43] + tj[J_ch3br]) + T(1));
    R[38] = -ck0[38] + x[38]*(F.dt*(K[K_e52]*x[42] + tj[J_h1211]) + T(1));
    R[41] = -ck0[41] + x[41]*(F.dt*(K[K_e54]*x[43] + tj[J_ch2br2]) + T(1));
    R[42] = x[42];
    R[43] = x[43];
    R[45] = x[45];
    R[49] = x[49];
    R[51] = x[51];
    R[56] = x[56];
    const T N_cno = nt_div<T>(K[K_b9]*x[46], K[K_b12]);
    const T N_dno = -N_cno + x[20];
    const bool sel_N_no2 = (N_dno) > (T(1e-30));
    const T N_no2 = sel_N_no2 ? T(N_dno) : T(nt_div<T>(T(1e-30)*x[20], N_cno + T(1e-30)));
    R[48] = -N_no2 + x[48];
    const bool sel_N_no3 = (N_dno) > (T(1e-30));
    const T N_no3 = sel_N_no3 ? T(N_cno) : T(nt_div<T>(N_cno*x[20], N_cno + T(1e-30)));
    R[54] = -N_no3 + x[54];
    const bool sel_N_bro = (x[23]) >= (T(0));
    const T N_bro = sel_N_bro ? T(x[23]) : T(T(0));
    R[53] = -N_bro + x[53];
}

// scaled Jacobian rows [0, 1, 4, 6, 14, 15, 18, 19, 21, 22, 23, 24, 25, 29, 30, 32, 34, 36, 38, 41, 42, 44, 46, 47, 48, 50, 55] (night equations) into their stored A slots
template <typename T, typename FF, typename PK, typename PJ>
__device__ __forceinline__ void nt_jacobian_night_w2_0(const FF& F, PK K, PK tj, PK het, const double* __restrict__ x, double floor_, PJ J) {
    const int fh = nt_exp_hi(floor_);
    const T xt0 = nt_cvt<T>(x[0]);
    const T xt1 = nt_cvt<T>(x[1]);
    const T xt2 = nt_cvt<T>(x[2]);
    const T xt3 = nt_cvt<T>(x[3]);
    const T xt4 = nt_cvt<T>(x[4]);
    const T xt5 = nt_cvt<T>(x[5]);
    const T xt6 = nt_cvt<T>(x[6]);
    const T xt7 = nt_cvt<T>(x[7]);
    const T xt8 = nt_cvt<T>(x[8]);
    const T xt9 = nt_cvt<T>(x[9]);
    const T xt10 = nt_cvt<T>(x[10]);
    const T xt11 = nt_cvt<T>(x[11]);
    const T xt12 = nt_cvt<T>(x[12]);
    const T xt13 = nt_cvt<T>(x[13]);
    const T xt14 = nt_cvt<T>(x[14]);
    const T xt15 = nt_cvt<T>(x[15]);
    const T xt16 = nt_cvt<T>(x[16]);
    const T xt17 = nt_cvt<T>(x[17]);
    const T xt18 = nt_cvt<T>(x[18]);
    const T xt19 = nt_cvt<T>(x[19]);
    const T xt20 = nt_cvt<T>(x[20]);
    const T xt21 = nt_cvt<T>(x[21]);
    const T xt22 = nt_cvt<T>(x[22]);
    const T xt23 = nt_cvt<T>(x[23]);
    const T xt24 = nt_cvt<T>(x[24]);
    const T xt25 = nt_cvt<T>(x[25]);
    const T xt26 = nt_cvt<T>(x[26]);
    const T xt27 = nt_cvt<T>(x[27]);
    const T xt28 = nt_cvt<T>(x[28]);
    const T xt29 = nt_cvt<T>(x[29]);
    const T xt30 = nt_cvt<T>(x[30]);
    const T xt31 = nt_cvt<T>(x[31]);
    const T xt32 = nt_cvt<T>(x[32]);
    const T xt33 = nt_cvt<T>(x[33]);
    const T xt34 = nt_cvt<T>(x[34]);
    const T xt35 = nt_cvt<T>(x[35]);
    const T xt36 = nt_cvt<T>(x[36]);
    const T xt37 = nt_cvt<T>(x[37]);
    const T xt38 = nt_cvt<T>(x[38]);
    const T xt39 = nt_cvt<T>(x[39]);
    const T xt40 = nt_cvt<T>(x[40]);
    const T xt41 = nt_cvt<T>(x[41]);
    const T xt42 = nt_cvt<T>(x[42]);
    const T xt43 = nt_cvt<T>(x[43]);
    const T xt44 = nt_cvt<T>(x[44]);
    const T xt45 = nt_cvt<T>(x[45]);
    const T xt46 = nt_cvt<T>(x[46]);
    const T xt47 = nt_cvt<T>(x[47]);
    const T xt48 = nt_cvt<T>(x[48]);
    const T xt49 = nt_cvt<T>(x[49]);
    const T xt50 = nt_cvt<T>(x[50]);
    const T xt51 = nt_cvt<T>(x[51]);
    const T xt52 = nt_cvt<T>(x[52]);
    const T xt53 = nt_cvt<T>(x[53]);
    const T xt54 = nt_cvt<T>(x[54]);
    const T xt55 = nt_cvt<T>(x[55]);
    const T xt56 = nt_cvt<T>(x[56]);
    const T cs0 = nt_scale<T>(nt_exp_hi(x[0]), fh);
    const T cs1 = nt_scale<T>(nt_exp_hi(x[1]), fh);
    const T cs2 = nt_scale<T>(nt_exp_hi(x[2]), fh);
    const T cs4 = nt_scale<T>(nt_exp_hi(x[4]), fh);
    const T cs5 = nt_scale<T>(nt_exp_hi(x[5]), fh);
    const T cs7 = nt_scale<T>(nt_exp_hi(x[7]), fh);
    const T cs8 = nt_scale<T>(nt_exp_hi(x[8]), fh);
    const T cs9 = nt_scale<T>(nt_exp_hi(x[9]), fh);
    const T cs12 = nt_scale<T>(nt_exp_hi(x[12]), fh);
    const T cs13 = nt_scale<T>(nt_exp_hi(x[13]), fh);
    const T cs14 = nt_scale<T>(nt_exp_hi(x[14]), fh);
    const T cs15 = nt_scale<T>(nt_exp_hi(x[15]), fh);
    const T cs16 = nt_scale<T>(nt_exp_hi(x[16]), fh);
    const T cs17 = nt_scale<T>(nt_exp_hi(x[17]), fh);
    const T cs18 = nt_scale<T>(nt_exp_hi(x[18]), fh);
    const T cs19 = nt_scale<T>(nt_exp_hi(x[19]), fh);
    const T cs20 = nt_scale<T>(nt_exp_hi(x[20]), fh);
    const T cs21 = nt_scale<T>(nt_exp_hi(x[21]), fh);
    const T cs24 = nt_scale<T>(nt_exp_hi(x[24]), fh);
    const T cs25 = nt_scale<T>(nt_exp_hi(x[25]), fh);
    const T cs26 = nt_scale<T>(nt_exp_hi(x[26]), fh);
    const T cs27 = nt_scale<T>(nt_exp_hi(x[27]), fh);
    const T cs28 = nt_scale<T>(nt_exp_hi(x[28]), fh);
    const T cs29 = nt_scale<T>(nt_exp_hi(x[29]), fh);
    const T cs30 = nt_scale<T>(nt_exp_hi(x[30]), fh);
    const T cs31 = nt_scale<T>(nt_exp_hi(x[31]), fh);
    const T cs32 = nt_scale<T>(nt_exp_hi(x[32]), fh);
    const T cs33 = nt_scale<T>(nt_exp_hi(x[33]), fh);
    const T cs34 = nt_scale<T>(nt_exp_hi(x[34]), fh);
    const T cs35 = nt_scale<T>(nt_exp_hi(x[35]), fh);
    const T cs36 = nt_scale<T>(nt_exp_hi(x[36]), fh);
    const T cs38 = nt_scale<T>(nt_exp_hi(x[38]), fh);
    const T cs41 = nt_scale<T>(nt_exp_hi(x[41]), fh);
    const T cs42 = nt_scale<T>(nt_exp_hi(x[42]), fh);
    const T cs43 = nt_scale<T>(nt_exp_hi(x[43]), fh);
    const T cs44 = nt_scale<T>(nt_exp_hi(x[44]), fh);
    const T cs45 = nt_scale<T>(nt_exp_hi(x[45]), fh);
    const T cs46 = nt_scale<T>(nt_exp_hi(x[46]), fh);
    const T cs47 = nt_scale<T>(nt_exp_hi(x[47]), fh);
    const T cs48 = nt_scale<T>(nt_exp_hi(x[48]), fh);
    const T cs49 = nt_scale<T>(nt_exp_hi(x[49]), fh);
    const T cs50 = nt_scale<T>(nt_exp_hi(x[50]), fh);
    const T cs52 = nt_scale<T>(nt_exp_hi(x[52]), fh);
    const T cs53 = nt_scale<T>(nt_exp_hi(x[53]), fh);
    const T cs55 = nt_scale<T>(nt_exp_hi(x[55]), fh);
    {  // row 0
    const T rs0 = nt_rscale<T>(nt_exp_hi(x[0]), fh);
        const T nj0_c0 = K[K_b38] + K[K_b39];
        J[76] = (F.dt*(nj0_c0*xt42 + tj[J_n2o]) + T(1)) * (cs0 * rs0);
        J[77] = (F.dt*nj0_c0*xt0) * (cs42 * rs0);
    }
    {  // row 1
    const T rs1 = nt_rscale<T>(nt_exp_hi(x[1]), fh);
        const T nj1_c0 = F.dt*xt1;
        J[157] = (F.dt*(K[K_c1a]*xt42 + K[K_c1b]*xt42 + K[K_c1c]*xt42 + K[K_c2]*xt43 + K[K_d5]*xt44) + T(1)) * (cs1 * rs1);
        J[156] = (nj1_c0*(K[K_c1a] + K[K_c1b] + K[K_c1c])) * (cs42 * rs1);
        J[159] = (K[K_c2]*nj1_c0) * (cs43 * rs1);
        J[158] = (K[K_d5]*nj1_c0) * (cs44 * rs1);
    }
    {  // row 4
    const T rs4 = nt_rscale<T>(nt_exp_hi(x[4]), fh);
        const T nj4_c0 = T(2)*het[2];
        const T nj4_c1 = F.dt*K[K_b22];
        J[122] = (-F.dt*(het[0]*xt13 + het[5]*xt19 + nj4_c0*xt5)) * (cs2 * rs4);
        J[120] = (F.dt*(F.parthno3*(K[K_b27]*xt43 + tj[J_hno3]) + F.rain_hno3) + T(1)) * (cs4 * rs4);
        J[118] = (-F.dt*(het[3]*xt12 + nj4_c0*xt2)) * (cs5 * rs4);
        J[121] = (-F.dt*(het[1]*xt13 + het[3]*xt5)) * (cs12 * rs4);
        J[119] = (-F.dt*(het[0]*xt2 + het[1]*xt12)) * (cs13 * rs4);
        J[117] = (-F.dt*het[5]*xt2) * (cs19 * rs4);
        J[124] = (F.dt*F.parthno3*K[K_b27]*xt4 - nj4_c1*xt48) * (cs43 * rs4);
        J[123] = (-nj4_c1*xt43) * (cs48 * rs4);
    }
    {  // row 6
    const T rs6 = nt_rscale<T>(nt_exp_hi(x[6]), fh);
        const T nj6_c0 = T(3)*xt42;
        const T nj6_c1 = T(2)*K[K_d91];
        const T nj6_c2 = T(4)*K[K_d93];
        const T nj6_c3 = T(3)*K[K_d94];
        J[9] = (F.dt*F.rain_hcl) * (cs12 * rs6);
        J[7] = (-F.dt*(K[K_d90]*nj6_c0 + T(3)*tj[J_cfc11])) * (cs30 * rs6);
        J[4] = (-F.dt*(nj6_c1*xt42 + T(2)*tj[J_cfc12])) * (cs31 * rs6);
        J[0] = (-F.dt*(K[K_d92]*nj6_c0 + T(3)*tj[J_cfc113])) * (cs32 * rs6);
        J[2] = (-F.dt*(nj6_c2*xt42 + T(4)*tj[J_ccl4])) * (cs33 * rs6);
        J[6] = (-F.dt*(nj6_c3*xt43 + T(3)*tj[J_ch3ccl3])) * (cs34 * rs6);
        J[5] = (-F.dt*(K[K_d95]*xt43 + tj[J_ch3cl])) * (cs35 * rs6);
        J[3] = (-F.dt*(K[K_d96]*xt42 + K[K_d97]*xt43 + tj[J_hcfc22])) * (cs36 * rs6);
        J[1] = (-F.dt*(K[K_e52]*xt42 + tj[J_h1211])) * (cs38 * rs6);
        J[8] = (-F.dt*(T(3)*K[K_d90]*xt30 + T(3)*K[K_d92]*xt32 + K[K_d96]*xt36 + K[K_e52]*xt38 + nj6_c1*xt31 + nj6_c2*xt33)) * (cs42 * rs6);
        J[10] = (-F.dt*(K[K_d95]*xt35 + K[K_d97]*xt36 + nj6_c3*xt34)) * (cs43 * rs6);
    }
    {  // row 14
    const T rs14 = nt_rscale<T>(nt_exp_hi(x[14]), fh);
        const T nj14_c0 = F.dt*het[0];
        const T nj14_c1 = F.dt*xt14;
        const T nj14_c2 = F.dt*K[K_d33];
        J[170] = (-nj14_c0*xt13) * (cs2 * rs14);
        J[169] = (het[4]*nj14_c1) * (cs12 * rs14);
        J[166] = (-nj14_c0*xt2) * (cs13 * rs14);
        J[167] = (F.dt*(K[K_d34]*xt43 + K[K_d35]*xt45 + K[K_d37]*xt44 + het[4]*xt12 + het[8]*xt18 + tj[J_hocl]) + T(1)) * (cs14 * rs14);
        J[168] = (het[8]*nj14_c1) * (cs18 * rs14);
        J[173] = (K[K_d34]*nj14_c1) * (cs43 * rs14);
        J[172] = (K[K_d37]*nj14_c1) * (cs44 * rs14);
        J[171] = (K[K_d35]*nj14_c1) * (cs45 * rs14);
        J[174] = (-nj14_c2*xt52) * (cs47 * rs14);
        J[175] = (-nj14_c2*xt47) * (cs52 * rs14);
    }
    {  // row 15
    const T rs15 = nt_rscale<T>(nt_exp_hi(x[15]), fh);
        J[63] = (-F.dt*(het[1]*xt13 + het[4]*xt14)) * (cs12 * rs15);
        J[61] = (-F.dt*het[1]*xt12) * (cs13 * rs15);
        J[62] = (-F.dt*(K[K_d37]*xt44 + het[4]*xt12)) * (cs14 * rs15);
        J[60] = (F.dt*tj[J_cl2] + T(1)) * (cs15 * rs15);
        J[64] = (-F.dt*K[K_d37]*xt14) * (cs44 * rs15);
        J[65] = (-T(2)*F.dt*K[K_d62]*xt52) * (cs52 * rs15);
    }
    {  // row 18
    const T rs18 = nt_rscale<T>(nt_exp_hi(x[18]), fh);
        const T nj18_c0 = F.dt*xt18;
        const T nj18_c1 = F.dt*xt50;
        const T nj18_c2 = F.parthbr*nj18_c0;
        J[183] = (het[8]*nj18_c0) * (cs14 * rs18);
        J[184] = (F.dt*(F.parthbr*(K[K_e11]*xt43 + K[K_e9]*xt42 + tj[J_hbr]) + F.rain_hbr + het[7]*xt25 + het[8]*xt14) + T(1)) * (cs18 * rs18);
        J[181] = (het[7]*nj18_c0) * (cs25 * rs18);
        J[185] = (-K[K_c19]*nj18_c1) * (cs27 * rs18);
        J[182] = (K[K_e9]*nj18_c2) * (cs42 * rs18);
        J[187] = (K[K_e11]*nj18_c2) * (cs43 * rs18);
        J[188] = (-K[K_e7]*nj18_c1) * (cs47 * rs18);
        J[186] = (-F.dt*(K[K_c19]*xt27 + K[K_e7]*xt47)) * (cs50 * rs18);
    }
    {  // row 19
    const T rs19 = nt_rscale<T>(nt_exp_hi(x[19]), fh);
        const T nj19_c0 = F.dt*xt19;
        const T nj19_c1 = F.dt*K[K_e13];
        J[56] = (het[5]*nj19_c0) * (cs2 * rs19);
        J[55] = (F.dt*(K[K_e8]*xt45 + het[5]*xt2 + tj[J_brono2]) + T(1)) * (cs19 * rs19);
        J[58] = (K[K_e8]*nj19_c0) * (cs45 * rs19);
        J[57] = (-nj19_c1*xt53) * (cs48 * rs19);
        J[59] = (-nj19_c1*xt48) * (cs53 * rs19);
    }
    {  // row 21
    const T rs21 = nt_rscale<T>(nt_exp_hi(x[21]), fh);
        const T nj21_c0 = F.dt*K[K_b23];
        J[152] = (F.dt*(F.hnm*K[K_b24] + K[K_b28]*xt43 + tj[J_hno4]) + T(1)) * (cs21 * rs21);
        J[154] = (F.dt*K[K_b28]*xt21) * (cs43 * rs21);
        J[155] = (-nj21_c0*xt48) * (cs47 * rs21);
        J[153] = (-nj21_c0*xt47) * (cs48 * rs21);
    }
    {  // row 22
    const T rs22 = nt_rscale<T>(nt_exp_hi(x[22]), fh);
        const T nj22_c0 = F.dt*xt44;
        const T nj22_c1 = T(3)*xt42;
        const T nj22_c2 = T(2)*K[K_d91];
        const T nj22_c3 = T(4)*K[K_d93];
        const T nj22_c4 = T(3)*K[K_d94];
        const T nj22_c5 = F.dt*xt52;
        const T nj22_c6 = T(2)*K[K_d60];
        const T nj22_c7 = T(2)*K[K_d62];
        J[141] = (K[K_d5]*nj22_c0) * (cs1 * rs22);
        J[140] = (-F.dt*tj[J_oclo]) * (cs9 * rs22);
        J[144] = (-F.dt*F.parthcl*(K[K_d11]*xt43 + tj[J_hcl])) * (cs12 * rs22);
        J[135] = (-F.dt*(K[K_d32]*xt45 + tj[J_clono2_cl] + tj[J_clono2_clo])) * (cs13 * rs22);
        J[142] = (-F.dt*(K[K_d34]*xt43 + K[K_d35]*xt45 + tj[J_hocl]) + K[K_d37]*nj22_c0) * (cs14 * rs22);
        J[133] = (-T(2)*F.dt*tj[J_cl2]) * (cs15 * rs22);
        J[128] = (-F.dt*tj[J_clno2]) * (cs17 * rs22);
        J[138] = (-F.dt*(T(2)*F.hnm*K[K_d61] + T(2)*tj[J_cl2o2])) * (cs24 * rs22);
        J[132] = (-F.dt*tj[J_brcl]) * (cs26 * rs22);
        J[143] = (K[K_c10]*nj22_c0) * (cs27 * rs22);
        J[137] = (-F.dt*(K[K_d90]*nj22_c1 + T(3)*tj[J_cfc11])) * (cs30 * rs22);
        J[131] = (-F.dt*(nj22_c2*xt42 + T(2)*tj[J_cfc12])) * (cs31 * rs22);
        J[127] = (-F.dt*(K[K_d92]*nj22_c1 + T(3)*tj[J_cfc113])) * (cs32 * rs22);
        J[129] = (-F.dt*(nj22_c3*xt42 + T(4)*tj[J_ccl4])) * (cs33 * rs22);
        J[136] = (-F.dt*(nj22_c4*xt43 + T(3)*tj[J_ch3ccl3])) * (cs34 * rs22);
        J[134] = (-F.dt*(K[K_d95]*xt43 + tj[J_ch3cl])) * (cs35 * rs22);
        J[130] = (-F.dt*(K[K_d96]*xt42 + K[K_d97]*xt43 + tj[J_hcfc22])) * (cs36 * rs22);
        J[139] = (-F.dt*(T(3)*K[K_d90]*xt30 + T(3)*K[K_d92]*xt32 + K[K_d96]*xt36 + nj22_c2*xt31 + nj22_c3*xt33)) * (cs42 * rs22);
        J[149] = (-F.dt*(F.parthcl*K[K_d11]*xt12 + K[K_d34]*xt14 + K[K_d95]*xt35 + K[K_d97]*xt36 + nj22_c4*xt34) + K[K_d9]*nj22_c5) * (cs43 * rs22);
        J[147] = (F.dt*(F.h2*K[K_d6] + K[K_c10]*xt27 + K[K_d36]*xt48 + K[K_d37]*xt14 + K[K_d5]*xt1 + K[K_d7]*xt47)) * (cs44 * rs22);
        J[146] = (-F.dt*(K[K_d32]*xt13 + K[K_d35]*xt14)) * (cs45 * rs22);
        J[150] = (F.dt*(K[K_d33]*xt52 + K[K_d7]*xt44)) * (cs47 * rs22);
        J[145] = (F.dt*(K[K_d31]*xt52 + K[K_d36]*xt44)) * (cs48 * rs22);
        J[151] = (F.dt*(K[K_d31]*xt48 + K[K_d33]*xt47 + K[K_d9]*xt43 + K[K_e5a]*xt53 + K[K_e5c]*xt53 + nj22_c6*xt52 + nj22_c7*xt52 + xt52*(nj22_c6 + nj22_c7))) * (cs52 * rs22);
        J[148] = (nj22_c5*(K[K_e5a] + K[K_e5c])) * (cs53 * rs22);
    }
    {  // row 23
    const T rs23 = nt_rscale<T>(nt_exp_hi(x[23]), fh);
        const T nj23_c0 = T(2)*het[7];
        const T nj23_c1 = F.dt*F.parthbr*xt18;
        const T nj23_c2 = F.dt*xt53;
        J[196] = (-F.dt*(F.parthbr*(K[K_e11]*xt43 + K[K_e9]*xt42 + tj[J_hbr]) + nj23_c0*xt25)) * (cs18 * rs23);
        J[193] = (-F.dt*(K[K_e8]*xt45 + tj[J_brono2])) * (cs19 * rs23);
        J[194] = (-F.dt*(K[K_e16]*xt45 + nj23_c0*xt18 + tj[J_hobr])) * (cs25 * rs23);
        J[192] = (-F.dt*tj[J_brcl]) * (cs26 * rs23);
        J[197] = (F.dt*K[K_c19]*xt50) * (cs27 * rs23);
        J[195] = (-K[K_e9]*nj23_c1) * (cs42 * rs23);
        J[202] = (-K[K_e11]*nj23_c1) * (cs43 * rs23);
        J[199] = (-F.dt*(K[K_e16]*xt25 + K[K_e8]*xt19)) * (cs45 * rs23);
        J[203] = (F.dt*(K[K_e15]*xt53 + K[K_e7]*xt50)) * (cs47 * rs23);
        J[198] = (K[K_e13]*nj23_c2) * (cs48 * rs23);
        J[201] = (F.dt*(K[K_c19]*xt27 + K[K_e7]*xt47)) * (cs50 * rs23);
        J[204] = (K[K_e5c]*nj23_c2) * (cs52 * rs23);
        J[200] = (F.dt*(K[K_e13]*xt48 + K[K_e15]*xt47 + K[K_e5c]*xt52)) * (cs53 * rs23);
    }
    {  // row 24
    const T rs24 = nt_rscale<T>(nt_exp_hi(x[24]), fh);
        J[97] = (F.dt*(F.hnm*K[K_d61] + tj[J_cl2o2]) + T(1)) * (cs24 * rs24);
        J[98] = (-T(2)*F.dt*K[K_d60]*xt52) * (cs52 * rs24);
    }
    {  // row 25
    const T rs25 = nt_rscale<T>(nt_exp_hi(x[25]), fh);
        const T nj25_c0 = F.dt*het[5];
        const T nj25_c1 = F.dt*xt25;
        const T nj25_c2 = F.dt*K[K_e15];
        J[83] = (-nj25_c0*xt19) * (cs2 * rs25);
        J[82] = (het[6]*nj25_c1) * (cs12 * rs25);
        J[81] = (het[7]*nj25_c1) * (cs18 * rs25);
        J[79] = (-nj25_c0*xt2) * (cs19 * rs25);
        J[80] = (F.dt*(K[K_e16]*xt45 + het[6]*xt12 + het[7]*xt18 + tj[J_hobr]) + T(1)) * (cs25 * rs25);
        J[84] = (K[K_e16]*nj25_c1) * (cs45 * rs25);
        J[86] = (-nj25_c2*xt53) * (cs47 * rs25);
        J[85] = (-nj25_c2*xt47) * (cs53 * rs25);
    }
    {  // row 29
    const T rs29 = nt_rscale<T>(nt_exp_hi(x[29]), fh);
        const T nj29_c0 = F.dt*K[K_c7];
        J[35] = (-nj29_c0*xt47) * (cs28 * rs29);
        J[34] = (F.dt*(K[K_c17a]*xt43 + K[K_c17b]*xt43 + tj[J_ch3o2h]) + T(1)) * (cs29 * rs29);
        J[36] = (F.dt*xt29*(K[K_c17a] + K[K_c17b])) * (cs43 * rs29);
        J[37] = (-nj29_c0*xt28) * (cs47 * rs29);
    }
    {  // row 30
    const T rs30 = nt_rscale<T>(nt_exp_hi(x[30]), fh);
        J[95] = (F.dt*(K[K_d90]*xt42 + tj[J_cfc11]) + T(1)) * (cs30 * rs30);
        J[96] = (F.dt*K[K_d90]*xt30) * (cs42 * rs30);
    }
    {  // row 32
    const T rs32 = nt_rscale<T>(nt_exp_hi(x[32]), fh);
        J[18] = (F.dt*(K[K_d92]*xt42 + tj[J_cfc113]) + T(1)) * (cs32 * rs32);
        J[19] = (F.dt*K[K_d92]*xt32) * (cs42 * rs32);
    }
    {  // row 34
    const T rs34 = nt_rscale<T>(nt_exp_hi(x[34]), fh);
        J[93] = (F.dt*(K[K_d94]*xt43 + tj[J_ch3ccl3]) + T(1)) * (cs34 * rs34);
        J[94] = (F.dt*K[K_d94]*xt34) * (cs43 * rs34);
    }
    {  // row 36
    const T rs36 = nt_rscale<T>(nt_exp_hi(x[36]), fh);
        const T nj36_c0 = F.dt*xt36;
        J[38] = (F.dt*(K[K_d96]*xt42 + K[K_d97]*xt43 + tj[J_hcfc22]) + T(1)) * (cs36 * rs36);
        J[39] = (K[K_d96]*nj36_c0) * (cs42 * rs36);
        J[40] = (K[K_d97]*nj36_c0) * (cs43 * rs36);
    }
    {  // row 38
    const T rs38 = nt_rscale<T>(nt_exp_hi(x[38]), fh);
        J[30] = (F.dt*(K[K_e52]*xt42 + tj[J_h1211]) + T(1)) * (cs38 * rs38);
        J[31] = (F.dt*K[K_e52]*xt38) * (cs42 * rs38);
    }
    {  // row 41
    const T rs41 = nt_rscale<T>(nt_exp_hi(x[41]), fh);
        J[125] = (F.dt*(K[K_e54]*xt43 + tj[J_ch2br2]) + T(1)) * (cs41 * rs41);
        J[126] = (F.dt*K[K_e54]*xt41) * (cs43 * rs41);
    }
    {  // row 42
    const T rs42 = nt_rscale<T>(nt_exp_hi(x[42]), fh);
        J[99] = T(0);
    }
    {  // row 44
    const T rs44 = nt_rscale<T>(nt_exp_hi(x[44]), fh);
        J[284] = T(0);
        J[288] = T(0);
        J[287] = T(0);
        J[285] = T(0);
        J[286] = T(0);
        J[292] = T(0);
        J[290] = T(0);
        J[294] = T(0);
        J[293] = T(0);
        J[289] = T(0);
        J[295] = T(0);
        J[296] = T(0);
        J[291] = T(0);
    }
    {  // row 46
    const T rs46 = nt_rscale<T>(nt_exp_hi(x[46]), fh);
        J[355] = (T(-1)) * (cs7 * rs46);
        J[358] = T(0);
        J[357] = T(0);
        J[359] = T(0);
        J[360] = T(0);
        J[356] = T(0);
    }
    {  // row 47
    const T rs47 = nt_rscale<T>(nt_exp_hi(x[47]), fh);
        J[342] = T(0);
        J[343] = T(0);
        J[345] = T(0);
        J[350] = T(0);
        J[347] = T(0);
        J[346] = T(0);
        J[352] = T(0);
        J[351] = (T(1)) * (cs47 * rs47);
        J[353] = T(0);
        J[349] = T(0);
        J[354] = T(0);
        J[348] = T(0);
        J[344] = T(0);
    }
    {  // row 50
    const T rs50 = nt_rscale<T>(nt_exp_hi(x[50]), fh);
        J[307] = T(0);
        J[311] = T(0);
        J[309] = T(0);
        J[313] = T(0);
        J[312] = T(0);
        J[308] = T(0);
        J[314] = T(0);
        J[315] = T(0);
        J[310] = T(0);
    }
    {  // row 55
    const T rs55 = nt_rscale<T>(nt_exp_hi(x[55]), fh);
        J[205] = T(0);
        J[207] = T(0);
        J[206] = T(0);
        J[209] = T(0);
        J[208] = T(0);
    }
    const T N_cno_c0 = nt_div<T>(K[K_b9], K[K_b12]);
    const T N_cno = N_cno_c0*xt46;
    const T d_N_cno_46 = N_cno_c0;
    const T N_dno = -N_cno + xt20;
    const T d_N_dno_20 = T(1);
    const T d_N_dno_46 = -d_N_cno_46;
    const T N_no2_c0 = N_cno + T(1e-30);
    const T N_no2_c1 = nt_div<T>(T(1e-30), N_no2_c0);
    const bool sel_N_no2 = (N_dno) > (T(1e-30));
    const T N_no2 = sel_N_no2 ? T(N_dno) : T(N_no2_c1*xt20);
    const T d_N_no2_20 = sel_N_no2 ? T(d_N_dno_20) : T(N_no2_c1);
    const T d_N_no2_46 = sel_N_no2 ? T(d_N_dno_46) : T(nt_div<T>(-T(1e-30)*d_N_cno_46*xt20, (N_no2_c0*N_no2_c0)));
    {  // row 48
    const T rs48 = nt_rscale<T>(nt_exp_hi(x[48]), fh);
        J[270] = (-d_N_no2_20) * (cs20 * rs48);
        J[269] = T(0);
        J[272] = T(0);
        J[275] = (-d_N_no2_46) * (cs46 * rs48);
        J[274] = T(0);
        J[271] = (T(1)) * (cs48 * rs48);
        J[276] = T(0);
        J[277] = T(0);
        J[273] = T(0);
    }
}

// residual rows [0, 1, 2, 5, 7, 9, 10, 12, 14, 17, 19, 20, 24, 25, 28, 29, 31, 33, 35, 36, 39, 40, 44, 46, 47, 50, 52, 55] (night equations, FP64)
template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>
__device__ __forceinline__ void nt_residual_night_w2_1(const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {
    R[0] = -ck0[0] + x[0]*(F.dt*(tj[J_n2o] + x[42]*(K[K_b38] + K[K_b39])) + T(1));
    R[1] = -ck0[1] + x[1]*(F.dt*(K[K_c1a]*x[42] + K[K_c1b]*x[42] + K[K_c1c]*x[42] + K[K_c2]*x[43] + K[K_d5]*x[44]) + T(1));
    const T nr2_c0 = x[29]*x[43];
    R[2] = -F.dt*(F.h2*K[K_a19]*x[43] + F.parthcl*K[K_d11]*x[12]*x[43] + F.parthno3*K[K_b27]*x[43]*x[4] + K[K_a30]*x[16]*x[43] + K[K_a31]*(x[43]*x[43]) + K[K_c17a]*nr2_c0 + K[K_c17b]*nr2_c0 + K[K_c2]*x[1]*x[43] + K[K_c8]*x[27]*x[43] + x[47]*(K[K_a17]*x[43] + T(1.6e-12)*x[55])) - ck0[2] + x[2]*(F.dt*F.parth2o*(K[K_a1et]*x[42] + tj[J_h2o]) + T(1));
    R[5] = -F.dt*K[K_b12]*x[48]*x[54] - ck0[5] + x[5]*(F.dt*(F.hnm*K[K_b32] + het[2]*x[2] + het[3]*x[12] + tj[J_n2o5]) + T(1));
    R[9] = -F.dt*K[K_e5a]*x[52]*x[53] - ck0[9] + x[9]*(F.dt*tj[J_oclo] + T(1));
    R[10] = -ck0[10] + x[10];
    R[12] = -F.dt*(K[K_d9]*x[43]*x[52] + x[44]*(F.h2*K[K_d6] + K[K_c10]*x[27] + K[K_d5]*x[1] + K[K_d7]*x[47])) - ck0[12] + x[12]*(F.dt*(F.parthcl*(K[K_d11]*x[43] + tj[J_hcl]) + F.rain_hcl + het[1]*x[13] + het[3]*x[5] + het[4]*x[14] + het[6]*x[25]) + T(1));
    R[14] = -F.dt*(K[K_d33]*x[47]*x[52] + het[0]*x[13]*x[2]) - ck0[14] + x[14]*(F.dt*(K[K_d34]*x[43] + K[K_d35]*x[45] + K[K_d37]*x[44] + het[4]*x[12] + het[8]*x[18] + tj[J_hocl]) + T(1));
    R[17] = -F.dt*(K[K_d36]*x[44]*x[48] + het[3]*x[12]*x[5]) - ck0[17] + x[17]*(F.dt*tj[J_clno2] + T(1));
    R[19] = -F.dt*K[K_e13]*x[48]*x[53] - ck0[19] + x[19]*(F.dt*(K[K_e8]*x[45] + het[5]*x[2] + tj[J_brono2]) + T(1));
    const T nr20_c0 = F.parthno3*x[4];
    R[20] = F.dt*(T(2)*K[K_b6]*x[49]*x[51] + x[48]*(T(2)*K[K_b12]*x[54] + K[K_b22]*x[43] + K[K_b23]*x[47] + K[K_d31]*x[52] + K[K_d36]*x[44] + K[K_e13]*x[53])) - F.dt*(K[K_b27]*nr20_c0*x[43] + T(2)*K[K_b39]*x[0]*x[42] + K[K_d32]*x[13]*x[45] + K[K_e8]*x[19]*x[45] + nr20_c0*tj[J_hno3] + tj[J_brono2]*x[19] + tj[J_clno2]*x[17] + x[13]*(tj[J_clono2_cl] + tj[J_clono2_clo]) + x[21]*(F.hnm*K[K_b24] + K[K_b28]*x[43] + tj[J_hno4]) + x[5]*(T(2)*F.hnm*K[K_b32] + T(2)*tj[J_n2o5])) - ck0[20] + x[20];
    R[24] = -F.dt*K[K_d60]*(x[52]*x[52]) - ck0[24] + x[24]*(F.dt*(F.hnm*K[K_d61] + tj[J_cl2o2]) + T(1));
    R[25] = -F.dt*(K[K_e15]*x[47]*x[53] + het[5]*x[19]*x[2]) - ck0[25] + x[25]*(F.dt*(K[K_e16]*x[45] + het[6]*x[12] + het[7]*x[18] + tj[J_hobr]) + T(1));
    R[28] = -F.dt*(F.o2*K[K_c4]*x[56] + K[K_c17a]*x[29]*x[43]) - ck0[28] + x[28]*(F.dt*(T(2)*K[K_c14]*x[28] + K[K_c18]*x[52] + K[K_c5]*x[49] + K[K_c7]*x[47]) + T(1));
    R[29] = -F.dt*K[K_c7]*x[28]*x[47] - ck0[29] + x[29]*(F.dt*(K[K_c17a]*x[43] + K[K_c17b]*x[43] + tj[J_ch3o2h]) + T(1));
    R[31] = -ck0[31] + x[31]*(F.dt*(K[K_d91]*x[42] + tj[J_cfc12]) + T(1));
    R[33] = -ck0[33] + x[33]*(F.dt*(K[K_d93]*x[42] + tj[J_ccl4]) + T(1));
    R[35] = -ck0[35] + x[35]*(F.dt*(K[K_d95]*x[43] + tj[J_ch3cl]) + T(1));
    R[36] = -ck0[36] + x[36]*(F.dt*(K[K_d96]*x[42] + K[K_d97]*x[43] + tj[J_hcfc22]) + T(1));
    R[39] = -ck0[39] + x[39]*(F.dt*(K[K_e53]*x[42] + tj[J_h1301]) + T(1));
    R[40] = F.dt*F.rain_hbr*x[18] - F.dt*(x[37]*(K[K_e50]*x[42] + K[K_e51]*x[43] + tj[J_ch3br]) + x[38]*(K[K_e52]*x[42] + tj[J_h1211]) + x[39]*(K[K_e53]*x[42] + tj[J_h1301]) + x[41]*(T(2)*K[K_e54]*x[43] + T(2)*tj[J_ch2br2])) - ck0[40] + x[40];
    R[44] = x[44];
    R[46] = x[46] - x[7];
    R[47] = x[47];
    R[50] = x[50];
    R[55] = x[55];
    const bool sel_N_clo = (x[22]) >= (T(0));
    const T N_clo = sel_N_clo ? T(x[22]) : T(T(0));
    R[52] = -N_clo + x[52];
    const T N_t06_c0 = tj[J_hocl]*x[14];
    const T N_t06_c1 = K[K_d33]*x[47]*x[52];
    const bool sel_N_t06 = (N_t06_c0) <= (N_t06_c1);
    const T N_t06 = sel_N_t06 ? T(N_t06_c0) : T(N_t06_c1);
    const T N_t07_c0 = K[K_e5c]*x[52]*x[53];
    const T N_t07_c1 = tj[J_brcl]*x[26];
    const bool sel_N_t07 = (N_t07_c0) <= (N_t07_c1);
    const T N_t07 = sel_N_t07 ? T(N_t07_c0) : T(N_t07_c1);
    const T N_t09_c0 = K[K_e15]*x[47]*x[53];
    const T N_t09_c1 = tj[J_hobr]*x[25];
    const bool sel_N_t09 = (N_t09_c0) <= (N_t09_c1);
    const T N_t09 = sel_N_t09 ? T(N_t09_c0) : T(N_t09_c1);
    const T nr7_c0 = T(2)*x[45];
    const T nr7_c1 = nt_div<T>(T(2)*tj[J_no3_no], fmax(T(1e-30), tj[J_no3_no2] + tj[J_no3_no]));
    R[7] = -F.dt*(T(2)*F.o2*tj[J_o2] + K[K_a26]*x[47]*x[49] + K[K_c5]*x[28]*x[49]) + F.dt*(K[K_b3]*nr7_c0*x[48] + K[K_b9]*nr7_c1*x[46]*x[48] + K[K_d3]*nr7_c0*x[52] + nt_div<T>(T(2)*K[K_d60]*tj[J_cl2o2]*(x[52]*x[52]), F.hnm*K[K_d61] + tj[J_cl2o2]) + T(2)*K[K_hk1]*(x[45]*x[45]) + K[K_hk3]*nr7_c0*x[46] + N_t06 + T(2)*N_t07 + N_t09 + nr7_c1*tj[J_clono2_cl]*x[13] + x[45]*(K[K_a5]*x[43] + K[K_a7]*x[47]) + x[46]*(K[K_a2]*x[55] + K[K_a6]*x[43] + K[K_a6b]*x[47])) - ck0[7] + x[7];
}

// scaled Jacobian rows [2, 3, 5, 7, 8, 9, 12, 13, 16, 17, 20, 26, 27, 28, 31, 33, 35, 37, 39, 40, 43, 45, 49, 51, 52, 53, 54, 56] (night equations) into their stored A slots
template <typename T, typename FF, typename PK, typename PJ>
__device__ __forceinline__ void nt_jacobian_night_w2_1(const FF& F, PK K, PK tj, PK het, const double* __restrict__ x, double floor_, PJ J) {
    const int fh = nt_exp_hi(floor_);
    const T xt0 = nt_cvt<T>(x[0]);
    const T xt1 = nt_cvt<T>(x[1]);
    const T xt2 = nt_cvt<T>(x[2]);
    const T xt3 = nt_cvt<T>(x[3]);
    const T xt4 = nt_cvt<T>(x[4]);
    const T xt5 = nt_cvt<T>(x[5]);
    const T xt6 = nt_cvt<T>(x[6]);
    const T xt7 = nt_cvt<T>(x[7]);
    const T xt8 = nt_cvt<T>(x[8]);
    const T xt9 = nt_cvt<T>(x[9]);
    const T xt10 = nt_cvt<T>(x[10]);
    const T xt11 = nt_cvt<T>(x[11]);
    const T xt12 = nt_cvt<T>(x[12]);
    const T xt13 = nt_cvt<T>(x[13]);
    const T xt14 = nt_cvt<T>(x[14]);
    const T xt15 = nt_cvt<T>(x[15]);
    const T xt16 = nt_cvt<T>(x[16]);
    const T xt17 = nt_cvt<T>(x[17]);
    const T xt18 = nt_cvt<T>(x[18]);
    const T xt19 = nt_cvt<T>(x[19]);
    const T xt20 = nt_cvt<T>(x[20]);
    const T xt21 = nt_cvt<T>(x[21]);
    const T xt22 = nt_cvt<T>(x[22]);
    const T xt23 = nt_cvt<T>(x[23]);
    const T xt24 = nt_cvt<T>(x[24]);
    const T xt25 = nt_cvt<T>(x[25]);
    const T xt26 = nt_cvt<T>(x[26]);
    const T xt27 = nt_cvt<T>(x[27]);
    const T xt28 = nt_cvt<T>(x[28]);
    const T xt29 = nt_cvt<T>(x[29]);
    const T xt30 = nt_cvt<T>(x[30]);
    const T xt31 = nt_cvt<T>(x[31]);
    const T xt32 = nt_cvt<T>(x[32]);
    const T xt33 = nt_cvt<T>(x[33]);
    const T xt34 = nt_cvt<T>(x[34]);
    const T xt35 = nt_cvt<T>(x[35]);
    const T xt36 = nt_cvt<T>(x[36]);
    const T xt37 = nt_cvt<T>(x[37]);
    const T xt38 = nt_cvt<T>(x[38]);
    const T xt39 = nt_cvt<T>(x[39]);
    const T xt40 = nt_cvt<T>(x[40]);
    const T xt41 = nt_cvt<T>(x[41]);
    const T xt42 = nt_cvt<T>(x[42]);
    const T xt43 = nt_cvt<T>(x[43]);
    const T xt44 = nt_cvt<T>(x[44]);
    const T xt45 = nt_cvt<T>(x[45]);
    const T xt46 = nt_cvt<T>(x[46]);
    const T xt47 = nt_cvt<T>(x[47]);
    const T xt48 = nt_cvt<T>(x[48]);
    const T xt49 = nt_cvt<T>(x[49]);
    const T xt50 = nt_cvt<T>(x[50]);
    const T xt51 = nt_cvt<T>(x[51]);
    const T xt52 = nt_cvt<T>(x[52]);
    const T xt53 = nt_cvt<T>(x[53]);
    const T xt54 = nt_cvt<T>(x[54]);
    const T xt55 = nt_cvt<T>(x[55]);
    const T xt56 = nt_cvt<T>(x[56]);
    const T cs0 = nt_scale<T>(nt_exp_hi(x[0]), fh);
    const T cs1 = nt_scale<T>(nt_exp_hi(x[1]), fh);
    const T cs2 = nt_scale<T>(nt_exp_hi(x[2]), fh);
    const T cs4 = nt_scale<T>(nt_exp_hi(x[4]), fh);
    const T cs5 = nt_scale<T>(nt_exp_hi(x[5]), fh);
    const T cs8 = nt_scale<T>(nt_exp_hi(x[8]), fh);
    const T cs9 = nt_scale<T>(nt_exp_hi(x[9]), fh);
    const T cs12 = nt_scale<T>(nt_exp_hi(x[12]), fh);
    const T cs13 = nt_scale<T>(nt_exp_hi(x[13]), fh);
    const T cs14 = nt_scale<T>(nt_exp_hi(x[14]), fh);
    const T cs16 = nt_scale<T>(nt_exp_hi(x[16]), fh);
    const T cs17 = nt_scale<T>(nt_exp_hi(x[17]), fh);
    const T cs18 = nt_scale<T>(nt_exp_hi(x[18]), fh);
    const T cs19 = nt_scale<T>(nt_exp_hi(x[19]), fh);
    const T cs20 = nt_scale<T>(nt_exp_hi(x[20]), fh);
    const T cs21 = nt_scale<T>(nt_exp_hi(x[21]), fh);
    const T cs22 = nt_scale<T>(nt_exp_hi(x[22]), fh);
    const T cs23 = nt_scale<T>(nt_exp_hi(x[23]), fh);
    const T cs25 = nt_scale<T>(nt_exp_hi(x[25]), fh);
    const T cs26 = nt_scale<T>(nt_exp_hi(x[26]), fh);
    const T cs27 = nt_scale<T>(nt_exp_hi(x[27]), fh);
    const T cs28 = nt_scale<T>(nt_exp_hi(x[28]), fh);
    const T cs29 = nt_scale<T>(nt_exp_hi(x[29]), fh);
    const T cs31 = nt_scale<T>(nt_exp_hi(x[31]), fh);
    const T cs33 = nt_scale<T>(nt_exp_hi(x[33]), fh);
    const T cs35 = nt_scale<T>(nt_exp_hi(x[35]), fh);
    const T cs37 = nt_scale<T>(nt_exp_hi(x[37]), fh);
    const T cs38 = nt_scale<T>(nt_exp_hi(x[38]), fh);
    const T cs39 = nt_scale<T>(nt_exp_hi(x[39]), fh);
    const T cs41 = nt_scale<T>(nt_exp_hi(x[41]), fh);
    const T cs42 = nt_scale<T>(nt_exp_hi(x[42]), fh);
    const T cs43 = nt_scale<T>(nt_exp_hi(x[43]), fh);
    const T cs44 = nt_scale<T>(nt_exp_hi(x[44]), fh);
    const T cs45 = nt_scale<T>(nt_exp_hi(x[45]), fh);
    const T cs46 = nt_scale<T>(nt_exp_hi(x[46]), fh);
    const T cs47 = nt_scale<T>(nt_exp_hi(x[47]), fh);
    const T cs48 = nt_scale<T>(nt_exp_hi(x[48]), fh);
    const T cs49 = nt_scale<T>(nt_exp_hi(x[49]), fh);
    const T cs50 = nt_scale<T>(nt_exp_hi(x[50]), fh);
    const T cs51 = nt_scale<T>(nt_exp_hi(x[51]), fh);
    const T cs52 = nt_scale<T>(nt_exp_hi(x[52]), fh);
    const T cs53 = nt_scale<T>(nt_exp_hi(x[53]), fh);
    const T cs54 = nt_scale<T>(nt_exp_hi(x[54]), fh);
    const T cs55 = nt_scale<T>(nt_exp_hi(x[55]), fh);
    const T cs56 = nt_scale<T>(nt_exp_hi(x[56]), fh);
    {  // row 2
    const T rs2 = nt_rscale<T>(nt_exp_hi(x[2]), fh);
        const T nj2_c0 = F.dt*xt43;
        const T nj2_c1 = F.dt*F.parth2o;
        const T nj2_c2 = F.parthno3*K[K_b27];
        const T nj2_c3 = F.parthcl*K[K_d11];
        J[261] = (-K[K_c2]*nj2_c0) * (cs1 * rs2);
        J[266] = (nj2_c1*(K[K_a1et]*xt42 + tj[J_h2o]) + T(1)) * (cs2 * rs2);
        J[260] = (-nj2_c0*nj2_c2) * (cs4 * rs2);
        J[265] = (-nj2_c0*nj2_c3) * (cs12 * rs2);
        J[262] = (-K[K_a30]*nj2_c0) * (cs16 * rs2);
        J[264] = (-K[K_c8]*nj2_c0) * (cs27 * rs2);
        J[258] = (-F.dt*(K[K_c17a]*xt43 + K[K_c17b]*xt43)) * (cs29 * rs2);
        J[259] = (K[K_a1et]*nj2_c1*xt2) * (cs42 * rs2);
        J[267] = (-F.dt*(F.h2*K[K_a19] + K[K_a17]*xt47 + K[K_a30]*xt16 + T(2)*K[K_a31]*xt43 + K[K_c17a]*xt29 + K[K_c17b]*xt29 + K[K_c2]*xt1 + K[K_c8]*xt27 + nj2_c2*xt4 + nj2_c3*xt12)) * (cs43 * rs2);
        J[268] = (-F.dt*(K[K_a17]*xt43 + T(1.6e-12)*xt55)) * (cs47 * rs2);
        J[263] = (-T(1.6e-12)*F.dt*xt47) * (cs55 * rs2);
    }
    {  // row 3
    const T rs3 = nt_rscale<T>(nt_exp_hi(x[3]), fh);
        const T nj3_c0 = T(2)*F.dt;
        const T nj3_c1 = K[K_b39]*nj3_c0;
        const T nj3_c2 = K[K_b6]*nj3_c0;
        J[20] = (-nj3_c1*xt42) * (cs0 * rs3);
        J[23] = (F.dt*F.rain_hno3) * (cs4 * rs3);
        J[22] = (-nj3_c1*xt0) * (cs42 * rs3);
        J[24] = (nj3_c2*xt51) * (cs49 * rs3);
        J[21] = (nj3_c2*xt49) * (cs51 * rs3);
    }
    {  // row 5
    const T rs5 = nt_rscale<T>(nt_exp_hi(x[5]), fh);
        const T nj5_c0 = F.dt*xt5;
        const T nj5_c1 = F.dt*K[K_b12];
        J[74] = (het[2]*nj5_c0) * (cs2 * rs5);
        J[72] = (F.dt*(F.hnm*K[K_b32] + het[2]*xt2 + het[3]*xt12 + tj[J_n2o5]) + T(1)) * (cs5 * rs5);
        J[73] = (het[3]*nj5_c0) * (cs12 * rs5);
        J[75] = (-nj5_c1*xt54) * (cs48 * rs5);
        J[71] = (-nj5_c1*xt48) * (cs54 * rs5);
    }
    {  // row 8
    const T rs8 = nt_rscale<T>(nt_exp_hi(x[8]), fh);
        const T nj8_c0 = F.dt*K[K_a36];
        J[160] = (nj8_c0*xt43 + T(1)) * (cs8 * rs8);
        J[161] = (-F.dt*tj[J_ch2o_co]) * (cs27 * rs8);
        J[165] = (nj8_c0*xt8) * (cs43 * rs8);
        J[163] = T(0);
        J[162] = T(0);
        J[164] = T(0);
    }
    {  // row 9
    const T rs9 = nt_rscale<T>(nt_exp_hi(x[9]), fh);
        const T nj9_c0 = F.dt*K[K_e5a];
        J[100] = (F.dt*tj[J_oclo] + T(1)) * (cs9 * rs9);
        J[102] = (-nj9_c0*xt53) * (cs52 * rs9);
        J[101] = (-nj9_c0*xt52) * (cs53 * rs9);
    }
    {  // row 12
    const T rs12 = nt_rscale<T>(nt_exp_hi(x[12]), fh);
        const T nj12_c0 = F.dt*xt44;
        const T nj12_c1 = F.dt*xt12;
        const T nj12_c2 = F.dt*K[K_d9];
        J[250] = (-K[K_d5]*nj12_c0) * (cs1 * rs12);
        J[247] = (het[3]*nj12_c1) * (cs5 * rs12);
        J[253] = (F.dt*(F.parthcl*(K[K_d11]*xt43 + tj[J_hcl]) + F.rain_hcl + het[1]*xt13 + het[3]*xt5 + het[4]*xt14 + het[6]*xt25) + T(1)) * (cs12 * rs12);
        J[249] = (het[1]*nj12_c1) * (cs13 * rs12);
        J[251] = (het[4]*nj12_c1) * (cs14 * rs12);
        J[248] = (het[6]*nj12_c1) * (cs25 * rs12);
        J[252] = (-K[K_c10]*nj12_c0) * (cs27 * rs12);
        J[255] = (F.parthcl*K[K_d11]*nj12_c1 - nj12_c2*xt52) * (cs43 * rs12);
        J[254] = (-F.dt*(F.h2*K[K_d6] + K[K_c10]*xt27 + K[K_d5]*xt1 + K[K_d7]*xt47)) * (cs44 * rs12);
        J[256] = (-K[K_d7]*nj12_c0) * (cs47 * rs12);
        J[257] = (-nj12_c2*xt43) * (cs52 * rs12);
    }
    {  // row 13
    const T rs13 = nt_rscale<T>(nt_exp_hi(x[13]), fh);
        const T nj13_c0 = F.dt*xt13;
        const T nj13_c1 = F.dt*K[K_d31];
        J[89] = (het[0]*nj13_c0) * (cs2 * rs13);
        J[88] = (het[1]*nj13_c0) * (cs12 * rs13);
        J[87] = (F.dt*(K[K_d32]*xt45 + het[0]*xt2 + het[1]*xt12 + tj[J_clono2_cl] + tj[J_clono2_clo]) + T(1)) * (cs13 * rs13);
        J[91] = (K[K_d32]*nj13_c0) * (cs45 * rs13);
        J[90] = (-nj13_c1*xt52) * (cs48 * rs13);
        J[92] = (-nj13_c1*xt48) * (cs52 * rs13);
    }
    {  // row 16
    const T rs16 = nt_rscale<T>(nt_exp_hi(x[16]), fh);
        J[189] = (F.dt*(F.rain_h2o2 + K[K_a30]*xt43 + tj[J_h2o2]) + T(1)) * (cs16 * rs16);
        J[190] = (F.dt*K[K_a30]*xt16) * (cs43 * rs16);
        J[191] = (-T(2)*F.dt*K[K_a27]*xt47) * (cs47 * rs16);
    }
    {  // row 17
    const T rs17 = nt_rscale<T>(nt_exp_hi(x[17]), fh);
        const T nj17_c0 = F.dt*het[3];
        const T nj17_c1 = F.dt*K[K_d36];
        J[26] = (-nj17_c0*xt12) * (cs5 * rs17);
        J[27] = (-nj17_c0*xt5) * (cs12 * rs17);
        J[25] = (F.dt*tj[J_clno2] + T(1)) * (cs17 * rs17);
        J[29] = (-nj17_c1*xt48) * (cs44 * rs17);
        J[28] = (-nj17_c1*xt44) * (cs48 * rs17);
    }
    {  // row 20
    const T rs20 = nt_rscale<T>(nt_exp_hi(x[20]), fh);
        const T nj20_c0 = T(2)*F.dt;
        const T nj20_c1 = K[K_b39]*nj20_c0;
        const T nj20_c2 = F.parthno3*K[K_b27];
        const T nj20_c3 = F.dt*xt48;
        const T nj20_c4 = T(2)*K[K_b12];
        const T nj20_c5 = K[K_b6]*nj20_c0;
        J[233] = (-nj20_c1*xt42) * (cs0 * rs20);
        J[237] = (-F.dt*(F.parthno3*tj[J_hno3] + nj20_c2*xt43)) * (cs4 * rs20);
        J[232] = (-F.dt*(T(2)*F.hnm*K[K_b32] + T(2)*tj[J_n2o5])) * (cs5 * rs20);
        J[235] = (-F.dt*(K[K_d32]*xt45 + tj[J_clono2_cl] + tj[J_clono2_clo])) * (cs13 * rs20);
        J[229] = (-F.dt*tj[J_clno2]) * (cs17 * rs20);
        J[230] = (-F.dt*(K[K_e8]*xt45 + tj[J_brono2])) * (cs19 * rs20);
        J[238] = (-F.dt*(F.hnm*K[K_b24] + K[K_b28]*xt43 + tj[J_hno4])) * (cs21 * rs20);
        J[236] = (-nj20_c1*xt0) * (cs42 * rs20);
        J[243] = (-F.dt*(K[K_b28]*xt21 + nj20_c2*xt4) + K[K_b22]*nj20_c3) * (cs43 * rs20);
        J[241] = (K[K_d36]*nj20_c3) * (cs44 * rs20);
        J[240] = (-F.dt*(K[K_d32]*xt13 + K[K_e8]*xt19)) * (cs45 * rs20);
        J[244] = (K[K_b23]*nj20_c3) * (cs47 * rs20);
        J[239] = (F.dt*(K[K_b22]*xt43 + K[K_b23]*xt47 + K[K_d31]*xt52 + K[K_d36]*xt44 + K[K_e13]*xt53 + nj20_c4*xt54)) * (cs48 * rs20);
        J[245] = (nj20_c5*xt51) * (cs49 * rs20);
        J[234] = (nj20_c5*xt49) * (cs51 * rs20);
        J[246] = (K[K_d31]*nj20_c3) * (cs52 * rs20);
        J[242] = (K[K_e13]*nj20_c3) * (cs53 * rs20);
        J[231] = (nj20_c3*nj20_c4) * (cs54 * rs20);
    }
    {  // row 26
    const T rs26 = nt_rscale<T>(nt_exp_hi(x[26]), fh);
        const T nj26_c0 = F.dt*het[6];
        const T nj26_c1 = F.dt*het[8];
        const T nj26_c2 = F.dt*K[K_e5c];
        J[47] = (-nj26_c0*xt25) * (cs12 * rs26);
        J[45] = (-nj26_c1*xt18) * (cs14 * rs26);
        J[46] = (-nj26_c1*xt14) * (cs18 * rs26);
        J[44] = (-nj26_c0*xt12) * (cs25 * rs26);
        J[43] = (F.dt*tj[J_brcl] + T(1)) * (cs26 * rs26);
        J[49] = (-nj26_c2*xt53) * (cs52 * rs26);
        J[48] = (-nj26_c2*xt52) * (cs53 * rs26);
    }
    {  // row 27
    const T rs27 = nt_rscale<T>(nt_exp_hi(x[27]), fh);
        const T nj27_c0 = F.dt*K[K_c1c];
        const T nj27_c1 = F.dt*K[K_c17b];
        const T nj27_c2 = F.dt*xt27;
        const T nj27_c3 = F.dt*K[K_c3];
        J[219] = (-nj27_c0*xt42) * (cs1 * rs27);
        J[222] = (F.dt*(K[K_c10]*xt44 + K[K_c19]*xt50 + K[K_c8]*xt43 + K[K_c9]*xt45 + tj[J_ch2o_co] + tj[J_ch2o_hco]) + T(1)) * (cs27 * rs27);
        J[221] = T(0);
        J[217] = (-nj27_c1*xt43) * (cs29 * rs27);
        J[218] = (-nj27_c0*xt1) * (cs42 * rs27);
        J[226] = (F.dt*K[K_c8]*xt27 - nj27_c1*xt29) * (cs43 * rs27);
        J[224] = (K[K_c10]*nj27_c2) * (cs44 * rs27);
        J[223] = (F.dt*K[K_c9]*xt27 - nj27_c3*xt56) * (cs45 * rs27);
        J[227] = T(0);
        J[225] = (K[K_c19]*nj27_c2) * (cs50 * rs27);
        J[228] = T(0);
        J[220] = (-nj27_c3*xt45) * (cs56 * rs27);
    }
    {  // row 28
    const T rs28 = nt_rscale<T>(nt_exp_hi(x[28]), fh);
        const T nj28_c0 = T(2)*K[K_c14]*xt28;
        const T nj28_c1 = F.dt*K[K_c17a];
        const T nj28_c2 = F.dt*xt28;
        J[212] = (F.dt*nj28_c0 + F.dt*(K[K_c18]*xt52 + K[K_c5]*xt49 + K[K_c7]*xt47 + nj28_c0) + T(1)) * (cs28 * rs28);
        J[210] = (-nj28_c1*xt43) * (cs29 * rs28);
        J[213] = (-nj28_c1*xt29) * (cs43 * rs28);
        J[214] = (K[K_c7]*nj28_c2) * (cs47 * rs28);
        J[215] = (K[K_c5]*nj28_c2) * (cs49 * rs28);
        J[216] = (K[K_c18]*nj28_c2) * (cs52 * rs28);
        J[211] = (-F.dt*F.o2*K[K_c4]) * (cs56 * rs28);
    }
    {  // row 31
    const T rs31 = nt_rscale<T>(nt_exp_hi(x[31]), fh);
        J[41] = (F.dt*(K[K_d91]*xt42 + tj[J_cfc12]) + T(1)) * (cs31 * rs31);
        J[42] = (F.dt*K[K_d91]*xt31) * (cs42 * rs31);
    }
    {  // row 33
    const T rs33 = nt_rscale<T>(nt_exp_hi(x[33]), fh);
        J[32] = (F.dt*(K[K_d93]*xt42 + tj[J_ccl4]) + T(1)) * (cs33 * rs33);
        J[33] = (F.dt*K[K_d93]*xt33) * (cs42 * rs33);
    }
    {  // row 35
    const T rs35 = nt_rscale<T>(nt_exp_hi(x[35]), fh);
        J[66] = (F.dt*(K[K_d95]*xt43 + tj[J_ch3cl]) + T(1)) * (cs35 * rs35);
        J[67] = (F.dt*K[K_d95]*xt35) * (cs43 * rs35);
    }
    {  // row 37
    const T rs37 = nt_rscale<T>(nt_exp_hi(x[37]), fh);
        const T nj37_c0 = F.dt*xt37;
        J[52] = (F.dt*(K[K_e50]*xt42 + K[K_e51]*xt43 + tj[J_ch3br]) + T(1)) * (cs37 * rs37);
        J[53] = (K[K_e50]*nj37_c0) * (cs42 * rs37);
        J[54] = (K[K_e51]*nj37_c0) * (cs43 * rs37);
    }
    {  // row 39
    const T rs39 = nt_rscale<T>(nt_exp_hi(x[39]), fh);
        J[50] = (F.dt*(K[K_e53]*xt42 + tj[J_h1301]) + T(1)) * (cs39 * rs39);
        J[51] = (F.dt*K[K_e53]*xt39) * (cs42 * rs39);
    }
    {  // row 40
    const T rs40 = nt_rscale<T>(nt_exp_hi(x[40]), fh);
        const T nj40_c0 = T(2)*K[K_e54];
        J[16] = (F.dt*F.rain_hbr) * (cs18 * rs40);
        J[13] = (-F.dt*(K[K_e50]*xt42 + K[K_e51]*xt43 + tj[J_ch3br])) * (cs37 * rs40);
        J[11] = (-F.dt*(K[K_e52]*xt42 + tj[J_h1211])) * (cs38 * rs40);
        J[12] = (-F.dt*(K[K_e53]*xt42 + tj[J_h1301])) * (cs39 * rs40);
        J[15] = (-F.dt*(nj40_c0*xt43 + T(2)*tj[J_ch2br2])) * (cs41 * rs40);
        J[14] = (-F.dt*(K[K_e50]*xt37 + K[K_e52]*xt38 + K[K_e53]*xt39)) * (cs42 * rs40);
        J[17] = (-F.dt*(K[K_e51]*xt37 + nj40_c0*xt41)) * (cs43 * rs40);
    }
    {  // row 43
    const T rs43 = nt_rscale<T>(nt_exp_hi(x[43]), fh);
        J[321] = T(0);
        J[331] = T(0);
        J[319] = T(0);
        J[322] = T(0);
        J[330] = T(0);
        J[323] = T(0);
        J[326] = T(0);
        J[325] = T(0);
        J[320] = T(0);
        J[317] = T(0);
        J[329] = T(0);
        J[328] = T(0);
        J[316] = T(0);
        J[318] = T(0);
        J[337] = (T(1)) * (cs43 * rs43);
        J[334] = T(0);
        J[333] = T(0);
        J[339] = T(0);
        J[338] = T(0);
        J[332] = T(0);
        J[340] = T(0);
        J[336] = T(0);
        J[341] = T(0);
        J[335] = T(0);
        J[327] = T(0);
        J[324] = T(0);
    }
    {  // row 45
    const T rs45 = nt_rscale<T>(nt_exp_hi(x[45]), fh);
        J[280] = T(0);
        J[279] = T(0);
        J[282] = T(0);
        J[281] = T(0);
        J[283] = T(0);
        J[278] = T(0);
    }
    {  // row 49
    const T rs49 = nt_rscale<T>(nt_exp_hi(x[49]), fh);
        J[361] = T(0);
        J[363] = T(0);
        J[366] = T(0);
        J[365] = T(0);
        J[362] = T(0);
        J[367] = T(0);
        J[364] = T(0);
    }
    {  // row 51
    const T rs51 = nt_rscale<T>(nt_exp_hi(x[51]), fh);
        J[78] = T(0);
    }
    {  // row 56
    const T rs56 = nt_rscale<T>(nt_exp_hi(x[56]), fh);
        J[177] = T(0);
        J[176] = T(0);
        J[180] = T(0);
        J[179] = T(0);
        J[178] = T(0);
    }
    const T N_cno_c0 = nt_div<T>(K[K_b9], K[K_b12]);
    const T N_cno = N_cno_c0*xt46;
    const T d_N_cno_46 = N_cno_c0;
    const T N_dno = -N_cno + xt20;
    const T d_N_dno_20 = T(1);
    const T d_N_dno_46 = -d_N_cno_46;
    const T N_no3_c0 = N_cno + T(1e-30);
    const T N_no3_c1 = nt_div<T>(T(1), N_no3_c0);
    const T N_no3_c2 = N_cno*N_no3_c1;
    const bool sel_N_no3 = (N_dno) > (T(1e-30));
    const T N_no3 = sel_N_no3 ? T(N_cno) : T(N_no3_c2*xt20);
    const T d_N_no3_20 = sel_N_no3 ? T(T(0)) : T(N_no3_c2);
    const T d_N_no3_46 = sel_N_no3 ? T(d_N_cno_46) : T(d_N_cno_46*(nt_div<T>(-N_cno*xt20, (N_no3_c0*N_no3_c0)) + N_no3_c1*xt20));
    {  // row 54
    const T rs54 = nt_rscale<T>(nt_exp_hi(x[54]), fh);
        J[68] = (-d_N_no3_20) * (cs20 * rs54);
        J[70] = (-d_N_no3_46) * (cs46 * rs54);
        J[69] = T(0);
    }
    const bool sel_N_clo = (xt22) >= (T(0));
    const T N_clo = sel_N_clo ? T(xt22) : T(T(0));
    const T d_N_clo_22 = sel_N_clo ? T(T(1)) : T(T(0));
    {  // row 52
    const T rs52 = nt_rscale<T>(nt_exp_hi(x[52]), fh);
        J[369] = T(0);
        J[373] = T(0);
        J[372] = T(0);
        J[370] = T(0);
        J[368] = (-d_N_clo_22) * (cs22 * rs52);
        J[371] = T(0);
        J[377] = T(0);
        J[375] = T(0);
        J[379] = T(0);
        J[378] = T(0);
        J[374] = T(0);
        J[380] = T(0);
        J[381] = (T(1)) * (cs52 * rs52);
        J[376] = T(0);
    }
    const bool sel_N_bro = (xt23) >= (T(0));
    const T N_bro = sel_N_bro ? T(xt23) : T(T(0));
    const T d_N_bro_23 = sel_N_bro ? T(T(1)) : T(T(0));
    {  // row 53
    const T rs53 = nt_rscale<T>(nt_exp_hi(x[53]), fh);
        J[297] = (-d_N_bro_23) * (cs23 * rs53);
        J[298] = T(0);
        J[302] = T(0);
        J[300] = T(0);
        J[304] = T(0);
        J[303] = T(0);
        J[299] = T(0);
        J[305] = T(0);
        J[306] = T(0);
        J[301] = (T(1)) * (cs53 * rs53);
    }
    const T N_t06_c0 = tj[J_hocl]*xt14;
    const T N_t06_c1 = K[K_d33]*xt52;
    const T N_t06_c2 = N_t06_c1*xt47;
    const bool sel_N_t06 = (N_t06_c0) <= (N_t06_c2);
    const T N_t06 = sel_N_t06 ? T(N_t06_c0) : T(N_t06_c2);
    const T d_N_t06_14 = sel_N_t06 ? T(tj[J_hocl]) : T(T(0));
    const T d_N_t06_47 = sel_N_t06 ? T(T(0)) : T(N_t06_c1);
    const T d_N_t06_52 = sel_N_t06 ? T(T(0)) : T(K[K_d33]*xt47);
    const T N_t07_c0 = K[K_e5c]*xt53;
    const T N_t07_c1 = N_t07_c0*xt52;
    const T N_t07_c2 = tj[J_brcl]*xt26;
    const bool sel_N_t07 = (N_t07_c1) <= (N_t07_c2);
    const T N_t07 = sel_N_t07 ? T(N_t07_c1) : T(N_t07_c2);
    const T d_N_t07_26 = sel_N_t07 ? T(T(0)) : T(tj[J_brcl]);
    const T d_N_t07_52 = sel_N_t07 ? T(N_t07_c0) : T(T(0));
    const T d_N_t07_53 = sel_N_t07 ? T(K[K_e5c]*xt52) : T(T(0));
    const T N_t09_c0 = K[K_e15]*xt53;
    const T N_t09_c1 = N_t09_c0*xt47;
    const T N_t09_c2 = tj[J_hobr]*xt25;
    const bool sel_N_t09 = (N_t09_c1) <= (N_t09_c2);
    const T N_t09 = sel_N_t09 ? T(N_t09_c1) : T(N_t09_c2);
    const T d_N_t09_25 = sel_N_t09 ? T(T(0)) : T(tj[J_hobr]);
    const T d_N_t09_47 = sel_N_t09 ? T(N_t09_c0) : T(T(0));
    const T d_N_t09_53 = sel_N_t09 ? T(K[K_e15]*xt47) : T(T(0));
    {  // row 7
    const T rs7 = nt_rscale<T>(nt_exp_hi(x[7]), fh);
        const T nj7_c0 = T(2)*F.dt;
        const T nj7_c1 = nt_div<T>(tj[J_no3_no], fmax(T(1e-30), tj[J_no3_no2] + tj[J_no3_no]));
        const T nj7_c2 = F.dt*xt49;
        const T nj7_c3 = T(2)*K[K_b3];
        const T nj7_c4 = T(2)*K[K_d3];
        const T nj7_c5 = T(2)*K[K_hk3];
        const T nj7_c6 = T(2)*K[K_b9]*nj7_c1;
        J[105] = (nj7_c0*nj7_c1*tj[J_clono2_cl]) * (cs13 * rs7);
        J[106] = (F.dt*d_N_t06_14) * (cs14 * rs7);
        J[104] = (F.dt*d_N_t09_25) * (cs25 * rs7);
        J[103] = (d_N_t07_26*nj7_c0) * (cs26 * rs7);
        J[108] = (-K[K_c5]*nj7_c2) * (cs28 * rs7);
        J[112] = (F.dt*(K[K_a5]*xt45 + K[K_a6]*xt46)) * (cs43 * rs7);
        J[110] = (F.dt*(K[K_a5]*xt43 + K[K_a7]*xt47 + T(4)*K[K_hk1]*xt45 + nj7_c3*xt48 + nj7_c4*xt52 + nj7_c5*xt46)) * (cs45 * rs7);
        J[114] = (F.dt*(K[K_a2]*xt55 + K[K_a6]*xt43 + K[K_a6b]*xt47 + nj7_c5*xt45 + nj7_c6*xt48)) * (cs46 * rs7);
        J[113] = (F.dt*d_N_t06_47 + F.dt*d_N_t09_47 + F.dt*(K[K_a6b]*xt46 + K[K_a7]*xt45) - K[K_a26]*nj7_c2) * (cs47 * rs7);
        J[109] = (F.dt*(nj7_c3*xt45 + nj7_c6*xt46)) * (cs48 * rs7);
        J[115] = (-F.dt*(K[K_a26]*xt47 + K[K_c5]*xt28)) * (cs49 * rs7);
        J[116] = (F.dt*d_N_t06_52 + F.dt*(nt_div<T>(T(4)*K[K_d60]*tj[J_cl2o2]*xt52, F.hnm*K[K_d61] + tj[J_cl2o2]) + nj7_c4*xt45) + d_N_t07_52*nj7_c0) * (cs52 * rs7);
        J[111] = (F.dt*d_N_t09_53 + d_N_t07_53*nj7_c0) * (cs53 * rs7);
        J[107] = (F.dt*K[K_a2]*xt46) * (cs55 * rs7);
    }
}

// residual rows of group g of 2 (night equations)
template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>
__device__ __forceinline__ void nt_residual_night_w2(int g, const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {
    switch (g) {
        case 0: nt_residual_night_w2_0<T>(F, K, tj, het, ck0, x, R); break;
        case 1: nt_residual_night_w2_1<T>(F, K, tj, het, ck0, x, R); break;
        default: break;
    }
}
// Jacobian rows of group g of 2 (night equations)
template <typename T, typename FF, typename PK, typename PJ>
__device__ __forceinline__ void nt_jacobian_night_w2(int g, const FF& F, PK K, PK tj, PK het, const double* __restrict__ x, double floor_, PJ J) {
    switch (g) {
        case 0: nt_jacobian_night_w2_0<T>(F, K, tj, het, x, floor_, J); break;
        case 1: nt_jacobian_night_w2_1<T>(F, K, tj, het, x, floor_, J); break;
        default: break;
    }
}

// residual rows [8, 9, 15, 21, 22, 26, 27, 33, 37, 39, 46, 47, 55] (night equations, FP64)
template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>
__device__ __forceinline__ void nt_residual_night_w4_0(const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {
    R[8] = -F.dt*(F.co2*tj[J_co2] + tj[J_ch2o_co]*x[27]) - ck0[8] + x[8]*(F.dt*K[K_a36]*x[43] + T(1));
    R[9] = -F.dt*K[K_e5a]*x[52]*x[53] - ck0[9] + x[9]*(F.dt*tj[J_oclo] + T(1));
    R[15] = -F.dt*(K[K_d37]*x[14]*x[44] + K[K_d62]*(x[52]*x[52]) + het[1]*x[12]*x[13] + het[4]*x[12]*x[14]) - ck0[15] + x[15]*(F.dt*tj[J_cl2] + T(1));
    R[21] = -F.dt*K[K_b23]*x[47]*x[48] - ck0[21] + x[21]*(F.dt*(F.hnm*K[K_b24] + K[K_b28]*x[43] + tj[J_hno4]) + T(1));
    const T nr22_c0 = T(2)*x[52];
    const T nr22_c1 = T(3)*x[42];
    R[22] = F.dt*(x[44]*(F.h2*K[K_d6] + K[K_c10]*x[27] + K[K_d36]*x[48] + K[K_d37]*x[14] + K[K_d5]*x[1] + K[K_d7]*x[47]) + x[52]*(K[K_d31]*x[48] + K[K_d33]*x[47] + K[K_d60]*nr22_c0 + K[K_d62]*nr22_c0 + K[K_d9]*x[43] + K[K_e5a]*x[53] + K[K_e5c]*x[53])) - F.dt*(F.parthcl*x[12]*(K[K_d11]*x[43] + tj[J_hcl]) + tj[J_brcl]*x[26] + T(2)*tj[J_cl2]*x[15] + tj[J_clno2]*x[17] + tj[J_oclo]*x[9] + x[13]*(K[K_d32]*x[45] + tj[J_clono2_cl] + tj[J_clono2_clo]) + x[14]*(K[K_d34]*x[43] + K[K_d35]*x[45] + tj[J_hocl]) + x[24]*(T(2)*F.hnm*K[K_d61] + T(2)*tj[J_cl2o2]) + x[30]*(K[K_d90]*nr22_c1 + T(3)*tj[J_cfc11]) + x[31]*(T(2)*K[K_d91]*x[42] + T(2)*tj[J_cfc12]) + x[32]*(K[K_d92]*nr22_c1 + T(3)*tj[J_cfc113]) + x[33]*(T(4)*K[K_d93]*x[42] + T(4)*tj[J_ccl4]) + x[34]*(T(3)*K[K_d94]*x[43] + T(3)*tj[J_ch3ccl3]) + x[35]*(K[K_d95]*x[43] + tj[J_ch3cl]) + x[36]*(K[K_d96]*x[42] + K[K_d97]*x[43] + tj[J_hcfc22])) - ck0[22] + x[22];
    R[26] = -F.dt*(K[K_e5c]*x[52]*x[53] + het[6]*x[12]*x[25] + het[8]*x[14]*x[18]) - ck0[26] + x[26]*(F.dt*tj[J_brcl] + T(1));
    R[27] = -F.dt*(K[K_c17b]*x[29]*x[43] + K[K_c1c]*x[1]*x[42] + K[K_c3]*x[45]*x[56]) - ck0[27] + x[27]*(F.dt*(K[K_c10]*x[44] + K[K_c19]*x[50] + K[K_c8]*x[43] + K[K_c9]*x[45] + tj[J_ch2o_co] + tj[J_ch2o_hco]) + T(1));
    R[33] = -ck0[33] + x[33]*(F.dt*(K[K_d93]*x[42] + tj[J_ccl4]) + T(1));
    R[37] = -ck0[37] + x[37]*(F.dt*(K[K_e50]*x[42] + K[K_e51]*x[43] + tj[J_ch3br]) + T(1));
    R[39] = -ck0[39] + x[39]*(F.dt*(K[K_e53]*x[42] + tj[J_h1301]) + T(1));
    R[46] = x[46] - x[7];
    R[47] = x[47];
    R[55] = x[55];
}

// scaled Jacobian rows [3, 9, 14, 21, 22, 25, 26, 31, 35, 43, 49, 52, 53, 56] (night equations) into their stored A slots
template <typename T, typename FF, typename PK, typename PJ>
__device__ __forceinline__ void nt_jacobian_night_w4_0(const FF& F, PK K, PK tj, PK het, const double* __restrict__ x, double floor_, PJ J) {
    const int fh = nt_exp_hi(floor_);
    const T xt0 = nt_cvt<T>(x[0]);
    const T xt1 = nt_cvt<T>(x[1]);
    const T xt2 = nt_cvt<T>(x[2]);
    const T xt3 = nt_cvt<T>(x[3]);
    const T xt4 = nt_cvt<T>(x[4]);
    const T xt5 = nt_cvt<T>(x[5]);
    const T xt6 = nt_cvt<T>(x[6]);
    const T xt7 = nt_cvt<T>(x[7]);
    const T xt8 = nt_cvt<T>(x[8]);
    const T xt9 = nt_cvt<T>(x[9]);
    const T xt10 = nt_cvt<T>(x[10]);
    const T xt11 = nt_cvt<T>(x[11]);
    const T xt12 = nt_cvt<T>(x[12]);
    const T xt13 = nt_cvt<T>(x[13]);
    const T xt14 = nt_cvt<T>(x[14]);
    const T xt15 = nt_cvt<T>(x[15]);
    const T xt16 = nt_cvt<T>(x[16]);
    const T xt17 = nt_cvt<T>(x[17]);
    const T xt18 = nt_cvt<T>(x[18]);
    const T xt19 = nt_cvt<T>(x[19]);
    const T xt20 = nt_cvt<T>(x[20]);
    const T xt21 = nt_cvt<T>(x[21]);
    const T xt22 = nt_cvt<T>(x[22]);
    const T xt23 = nt_cvt<T>(x[23]);
    const T xt24 = nt_cvt<T>(x[24]);
    const T xt25 = nt_cvt<T>(x[25]);
    const T xt26 = nt_cvt<T>(x[26]);
    const T xt27 = nt_cvt<T>(x[27]);
    const T xt28 = nt_cvt<T>(x[28]);
    const T xt29 = nt_cvt<T>(x[29]);
    const T xt30 = nt_cvt<T>(x[30]);
    const T xt31 = nt_cvt<T>(x[31]);
    const T xt32 = nt_cvt<T>(x[32]);
    const T xt33 = nt_cvt<T>(x[33]);
    const T xt34 = nt_cvt<T>(x[34]);
    const T xt35 = nt_cvt<T>(x[35]);
    const T xt36 = nt_cvt<T>(x[36]);
    const T xt37 = nt_cvt<T>(x[37]);
    const T xt38 = nt_cvt<T>(x[38]);
    const T xt39 = nt_cvt<T>(x[39]);
    const T xt40 = nt_cvt<T>(x[40]);
    const T xt41 = nt_cvt<T>(x[41]);
    const T xt42 = nt_cvt<T>(x[42]);
    const T xt43 = nt_cvt<T>(x[43]);
    const T xt44 = nt_cvt<T>(x[44]);
    const T xt45 = nt_cvt<T>(x[45]);
    const T xt46 = nt_cvt<T>(x[46]);
    const T xt47 = nt_cvt<T>(x[47]);
    const T xt48 = nt_cvt<T>(x[48]);
    const T xt49 = nt_cvt<T>(x[49]);
    const T xt50 = nt_cvt<T>(x[50]);
    const T xt51 = nt_cvt<T>(x[51]);
    const T xt52 = nt_cvt<T>(x[52]);
    const T xt53 = nt_cvt<T>(x[53]);
    const T xt54 = nt_cvt<T>(x[54]);
    const T xt55 = nt_cvt<T>(x[55]);
    const T xt56 = nt_cvt<T>(x[56]);
    const T cs0 = nt_scale<T>(nt_exp_hi(x[0]), fh);
    const T cs1 = nt_scale<T>(nt_exp_hi(x[1]), fh);
    const T cs2 = nt_scale<T>(nt_exp_hi(x[2]), fh);
    const T cs4 = nt_scale<T>(nt_exp_hi(x[4]), fh);
    const T cs8 = nt_scale<T>(nt_exp_hi(x[8]), fh);
    const T cs9 = nt_scale<T>(nt_exp_hi(x[9]), fh);
    const T cs12 = nt_scale<T>(nt_exp_hi(x[12]), fh);
    const T cs13 = nt_scale<T>(nt_exp_hi(x[13]), fh);
    const T cs14 = nt_scale<T>(nt_exp_hi(x[14]), fh);
    const T cs15 = nt_scale<T>(nt_exp_hi(x[15]), fh);
    const T cs16 = nt_scale<T>(nt_exp_hi(x[16]), fh);
    const T cs17 = nt_scale<T>(nt_exp_hi(x[17]), fh);
    const T cs18 = nt_scale<T>(nt_exp_hi(x[18]), fh);
    const T cs19 = nt_scale<T>(nt_exp_hi(x[19]), fh);
    const T cs21 = nt_scale<T>(nt_exp_hi(x[21]), fh);
    const T cs22 = nt_scale<T>(nt_exp_hi(x[22]), fh);
    const T cs23 = nt_scale<T>(nt_exp_hi(x[23]), fh);
    const T cs24 = nt_scale<T>(nt_exp_hi(x[24]), fh);
    const T cs25 = nt_scale<T>(nt_exp_hi(x[25]), fh);
    const T cs26 = nt_scale<T>(nt_exp_hi(x[26]), fh);
    const T cs27 = nt_scale<T>(nt_exp_hi(x[27]), fh);
    const T cs28 = nt_scale<T>(nt_exp_hi(x[28]), fh);
    const T cs29 = nt_scale<T>(nt_exp_hi(x[29]), fh);
    const T cs30 = nt_scale<T>(nt_exp_hi(x[30]), fh);
    const T cs31 = nt_scale<T>(nt_exp_hi(x[31]), fh);
    const T cs32 = nt_scale<T>(nt_exp_hi(x[32]), fh);
    const T cs33 = nt_scale<T>(nt_exp_hi(x[33]), fh);
    const T cs34 = nt_scale<T>(nt_exp_hi(x[34]), fh);
    const T cs35 = nt_scale<T>(nt_exp_hi(x[35]), fh);
    const T cs36 = nt_scale<T>(nt_exp_hi(x[36]), fh);
    const T cs42 = nt_scale<T>(nt_exp_hi(x[42]), fh);
    const T cs43 = nt_scale<T>(nt_exp_hi(x[43]), fh);
    const T cs44 = nt_scale<T>(nt_exp_hi(x[44]), fh);
    const T cs45 = nt_scale<T>(nt_exp_hi(x[45]), fh);
    const T cs46 = nt_scale<T>(nt_exp_hi(x[46]), fh);
    const T cs47 = nt_scale<T>(nt_exp_hi(x[47]), fh);
    const T cs48 = nt_scale<T>(nt_exp_hi(x[48]), fh);
    const T cs49 = nt_scale<T>(nt_exp_hi(x[49]), fh);
    const T cs50 = nt_scale<T>(nt_exp_hi(x[50]), fh);
    const T cs51 = nt_scale<T>(nt_exp_hi(x[51]), fh);
    const T cs52 = nt_scale<T>(nt_exp_hi(x[52]), fh);
    const T cs53 = nt_scale<T>(nt_exp_hi(x[53]), fh);
    const T cs55 = nt_scale<T>(nt_exp_hi(x[55]), fh);
    const T cs56 = nt_scale<T>(nt_exp_hi(x[56]), fh);
    {  // row 3
    const T rs3 = nt_rscale<T>(nt_exp_hi(x[3]), fh);
        const T nj3_c0 = T(2)*F.dt;
        const T nj3_c1 = K[K_b39]*nj3_c0;
        const T nj3_c2 = K[K_b6]*nj3_c0;
        J[20] = (-nj3_c1*xt42) * (cs0 * rs3);
        J[23] = (F.dt*F.rain_hno3) * (cs4 * rs3);
        J[22] = (-nj3_c1*xt0) * (cs42 * rs3);
        J[24] = (nj3_c2*xt51) * (cs49 * rs3);
        J[21] = (nj3_c2*xt49) * (cs51 * rs3);
    }
    {  // row 9
    const T rs9 = nt_rscale<T>(nt_exp_hi(x[9]), fh);
        const T nj9_c0 = F.dt*K[K_e5a];
        J[100] = (F.dt*tj[J_oclo] + T(1)) * (cs9 * rs9);
        J[102] = (-nj9_c0*xt53) * (cs52 * rs9);
        J[101] = (-nj9_c0*xt52) * (cs53 * rs9);
    }
    {  // row 14
    const T rs14 = nt_rscale<T>(nt_exp_hi(x[14]), fh);
        const T nj14_c0 = F.dt*het[0];
        const T nj14_c1 = F.dt*xt14;
        const T nj14_c2 = F.dt*K[K_d33];
        J[170] = (-nj14_c0*xt13) * (cs2 * rs14);
        J[169] = (het[4]*nj14_c1) * (cs12 * rs14);
        J[166] = (-nj14_c0*xt2) * (cs13 * rs14);
        J[167] = (F.dt*(K[K_d34]*xt43 + K[K_d35]*xt45 + K[K_d37]*xt44 + het[4]*xt12 + het[8]*xt18 + tj[J_hocl]) + T(1)) * (cs14 * rs14);
        J[168] = (het[8]*nj14_c1) * (cs18 * rs14);
        J[173] = (K[K_d34]*nj14_c1) * (cs43 * rs14);
        J[172] = (K[K_d37]*nj14_c1) * (cs44 * rs14);
        J[171] = (K[K_d35]*nj14_c1) * (cs45 * rs14);
        J[174] = (-nj14_c2*xt52) * (cs47 * rs14);
        J[175] = (-nj14_c2*xt47) * (cs52 * rs14);
    }
    {  // row 21
    const T rs21 = nt_rscale<T>(nt_exp_hi(x[21]), fh);
        const T nj21_c0 = F.dt*K[K_b23];
        J[152] = (F.dt*(F.hnm*K[K_b24] + K[K_b28]*xt43 + tj[J_hno4]) + T(1)) * (cs21 * rs21);
        J[154] = (F.dt*K[K_b28]*xt21) * (cs43 * rs21);
        J[155] = (-nj21_c0*xt48) * (cs47 * rs21);
        J[153] = (-nj21_c0*xt47) * (cs48 * rs21);
    }
    {  // row 22
    const T rs22 = nt_rscale<T>(nt_exp_hi(x[22]), fh);
        const T nj22_c0 = F.dt*xt44;
        const T nj22_c1 = T(3)*xt42;
        const T nj22_c2 = T(2)*K[K_d91];
        const T nj22_c3 = T(4)*K[K_d93];
        const T nj22_c4 = T(3)*K[K_d94];
        const T nj22_c5 = F.dt*xt52;
        const T nj22_c6 = T(2)*K[K_d60];
        const T nj22_c7 = T(2)*K[K_d62];
        J[141] = (K[K_d5]*nj22_c0) * (cs1 * rs22);
        J[140] = (-F.dt*tj[J_oclo]) * (cs9 * rs22);
        J[144] = (-F.dt*F.parthcl*(K[K_d11]*xt43 + tj[J_hcl])) * (cs12 * rs22);
        J[135] = (-F.dt*(K[K_d32]*xt45 + tj[J_clono2_cl] + tj[J_clono2_clo])) * (cs13 * rs22);
        J[142] = (-F.dt*(K[K_d34]*xt43 + K[K_d35]*xt45 + tj[J_hocl]) + K[K_d37]*nj22_c0) * (cs14 * rs22);
        J[133] = (-T(2)*F.dt*tj[J_cl2]) * (cs15 * rs22);
        J[128] = (-F.dt*tj[J_clno2]) * (cs17 * rs22);
        J[138] = (-F.dt*(T(2)*F.hnm*K[K_d61] + T(2)*tj[J_cl2o2])) * (cs24 * rs22);
        J[132] = (-F.dt*tj[J_brcl]) * (cs26 * rs22);
        J[143] = (K[K_c10]*nj22_c0) * (cs27 * rs22);
        J[137] = (-F.dt*(K[K_d90]*nj22_c1 + T(3)*tj[J_cfc11])) * (cs30 * rs22);
        J[131] = (-F.dt*(nj22_c2*xt42 + T(2)*tj[J_cfc12])) * (cs31 * rs22);
        J[127] = (-F.dt*(K[K_d92]*nj22_c1 + T(3)*tj[J_cfc113])) * (cs32 * rs22);
        J[129] = (-F.dt*(nj22_c3*xt42 + T(4)*tj[J_ccl4])) * (cs33 * rs22);
        J[136] = (-F.dt*(nj22_c4*xt43 + T(3)*tj[J_ch3ccl3])) * (cs34 * rs22);
        J[134] = (-F.dt*(K[K_d95]*xt43 + tj[J_ch3cl])) * (cs35 * rs22);
        J[130] = (-F.dt*(K[K_d96]*xt42 + K[K_d97]*xt43 + tj[J_hcfc22])) * (cs36 * rs22);
        J[139] = (-F.dt*(T(3)*K[K_d90]*xt30 + T(3)*K[K_d92]*xt32 + K[K_d96]*xt36 + nj22_c2*xt31 + nj22_c3*xt33)) * (cs42 * rs22);
        J[149] = (-F.dt*(F.parthcl*K[K_d11]*xt12 + K[K_d34]*xt14 + K[K_d95]*xt35 + K[K_d97]*xt36 + nj22_c4*xt34) + K[K_d9]*nj22_c5) * (cs43 * rs22);
        J[147] = (F.dt*(F.h2*K[K_d6] + K[K_c10]*xt27 + K[K_d36]*xt48 + K[K_d37]*xt14 + K[K_d5]*xt1 + K[K_d7]*xt47)) * (cs44 * rs22);
        J[146] = (-F.dt*(K[K_d32]*xt13 + K[K_d35]*xt14)) * (cs45 * rs22);
        J[150] = (F.dt*(K[K_d33]*xt52 + K[K_d7]*xt44)) * (cs47 * rs22);
        J[145] = (F.dt*(K[K_d31]*xt52 + K[K_d36]*xt44)) * (cs48 * rs22);
        J[151] = (F.dt*(K[K_d31]*xt48 + K[K_d33]*xt47 + K[K_d9]*xt43 + K[K_e5a]*xt53 + K[K_e5c]*xt53 + nj22_c6*xt52 + nj22_c7*xt52 + xt52*(nj22_c6 + nj22_c7))) * (cs52 * rs22);
        J[148] = (nj22_c5*(K[K_e5a] + K[K_e5c])) * (cs53 * rs22);
    }
    {  // row 25
    const T rs25 = nt_rscale<T>(nt_exp_hi(x[25]), fh);
        const T nj25_c0 = F.dt*het[5];
        const T nj25_c1 = F.dt*xt25;
        const T nj25_c2 = F.dt*K[K_e15];
        J[83] = (-nj25_c0*xt19) * (cs2 * rs25);
        J[82] = (het[6]*nj25_c1) * (cs12 * rs25);
        J[81] = (het[7]*nj25_c1) * (cs18 * rs25);
        J[79] = (-nj25_c0*xt2) * (cs19 * rs25);
        J[80] = (F.dt*(K[K_e16]*xt45 + het[6]*xt12 + het[7]*xt18 + tj[J_hobr]) + T(1)) * (cs25 * rs25);
        J[84] = (K[K_e16]*nj25_c1) * (cs45 * rs25);
        J[86] = (-nj25_c2*xt53) * (cs47 * rs25);
        J[85] = (-nj25_c2*xt47) * (cs53 * rs25);
    }
    {  // row 26
    const T rs26 = nt_rscale<T>(nt_exp_hi(x[26]), fh);
        const T nj26_c0 = F.dt*het[6];
        const T nj26_c1 = F.dt*het[8];
        const T nj26_c2 = F.dt*K[K_e5c];
        J[47] = (-nj26_c0*xt25) * (cs12 * rs26);
        J[45] = (-nj26_c1*xt18) * (cs14 * rs26);
        J[46] = (-nj26_c1*xt14) * (cs18 * rs26);
        J[44] = (-nj26_c0*xt12) * (cs25 * rs26);
        J[43] = (F.dt*tj[J_brcl] + T(1)) * (cs26 * rs26);
        J[49] = (-nj26_c2*xt53) * (cs52 * rs26);
        J[48] = (-nj26_c2*xt52) * (cs53 * rs26);
    }
    {  // row 31
    const T rs31 = nt_rscale<T>(nt_exp_hi(x[31]), fh);
        J[41] = (F.dt*(K[K_d91]*xt42 + tj[J_cfc12]) + T(1)) * (cs31 * rs31);
        J[42] = (F.dt*K[K_d91]*xt31) * (cs42 * rs31);
    }
    {  // row 35
    const T rs35 = nt_rscale<T>(nt_exp_hi(x[35]), fh);
        J[66] = (F.dt*(K[K_d95]*xt43 + tj[J_ch3cl]) + T(1)) * (cs35 * rs35);
        J[67] = (F.dt*K[K_d95]*xt35) * (cs43 * rs35);
    }
    {  // row 43
    const T rs43 = nt_rscale<T>(nt_exp_hi(x[43]), fh);
        J[321] = T(0);
        J[331] = T(0);
        J[319] = T(0);
        J[322] = T(0);
        J[330] = T(0);
        J[323] = T(0);
        J[326] = T(0);
        J[325] = T(0);
        J[320] = T(0);
        J[317] = T(0);
        J[329] = T(0);
        J[328] = T(0);
        J[316] = T(0);
        J[318] = T(0);
        J[337] = (T(1)) * (cs43 * rs43);
        J[334] = T(0);
        J[333] = T(0);
        J[339] = T(0);
        J[338] = T(0);
        J[332] = T(0);
        J[340] = T(0);
        J[336] = T(0);
        J[341] = T(0);
        J[335] = T(0);
        J[327] = T(0);
        J[324] = T(0);
    }
    {  // row 49
    const T rs49 = nt_rscale<T>(nt_exp_hi(x[49]), fh);
        J[361] = T(0);
        J[363] = T(0);
        J[366] = T(0);
        J[365] = T(0);
        J[362] = T(0);
        J[367] = T(0);
        J[364] = T(0);
    }
    {  // row 56
    const T rs56 = nt_rscale<T>(nt_exp_hi(x[56]), fh);
        J[177] = T(0);
        J[176] = T(0);
        J[180] = T(0);
        J[179] = T(0);
        J[178] = T(0);
    }
    const bool sel_N_clo = (xt22) >= (T(0));
    const T N_clo = sel_N_clo ? T(xt22) : T(T(0));
    const T d_N_clo_22 = sel_N_clo ? T(T(1)) : T(T(0));
    {  // row 52
    const T rs52 = nt_rscale<T>(nt_exp_hi(x[52]), fh);
        J[369] = T(0);
        J[373] = T(0);
        J[372] = T(0);
        J[370] = T(0);
        J[368] = (-d_N_clo_22) * (cs22 * rs52);
        J[371] = T(0);
        J[377] = T(0);
        J[375] = T(0);
        J[379] = T(0);
        J[378] = T(0);
        J[374] = T(0);
        J[380] = T(0);
        J[381] = (T(1)) * (cs52 * rs52);
        J[376] = T(0);
    }
    const bool sel_N_bro = (xt23) >= (T(0));
    const T N_bro = sel_N_bro ? T(xt23) : T(T(0));
    const T d_N_bro_23 = sel_N_bro ? T(T(1)) : T(T(0));
    {  // row 53
    const T rs53 = nt_rscale<T>(nt_exp_hi(x[53]), fh);
        J[297] = (-d_N_bro_23) * (cs23 * rs53);
        J[298] = T(0);
        J[302] = T(0);
        J[300] = T(0);
        J[304] = T(0);
        J[303] = T(0);
        J[299] = T(0);
        J[305] = T(0);
        J[306] = T(0);
        J[301] = (T(1)) * (cs53 * rs53);
    }
}

// residual rows [1, 7, 12, 14, 24, 25, 29, 31, 34, 36, 41, 42, 43, 49, 56] (night equations, FP64)
template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>
__device__ __forceinline__ void nt_residual_night_w4_1(const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {
    R[1] = -ck0[1] + x[1]*(F.dt*(K[K_c1a]*x[42] + K[K_c1b]*x[42] + K[K_c1c]*x[42] + K[K_c2]*x[43] + K[K_d5]*x[44]) + T(1));
    R[12] = -F.dt*(K[K_d9]*x[43]*x[52] + x[44]*(F.h2*K[K_d6] + K[K_c10]*x[27] + K[K_d5]*x[1] + K[K_d7]*x[47])) - ck0[12] + x[12]*(F.dt*(F.parthcl*(K[K_d11]*x[43] + tj[J_hcl]) + F.rain_hcl + het[1]*x[13] + het[3]*x[5] + het[4]*x[14] + het[6]*x[25]) + T(1));
    R[14] = -F.dt*(K[K_d33]*x[47]*x[52] + het[0]*x[13]*x[2]) - ck0[14] + x[14]*(F.dt*(K[K_d34]*x[43] + K[K_d35]*x[45] + K[K_d37]*x[44] + het[4]*x[12] + het[8]*x[18] + tj[J_hocl]) + T(1));
    R[24] = -F.dt*K[K_d60]*(x[52]*x[52]) - ck0[24] + x[24]*(F.dt*(F.hnm*K[K_d61] + tj[J_cl2o2]) + T(1));
    R[25] = -F.dt*(K[K_e15]*x[47]*x[53] + het[5]*x[19]*x[2]) - ck0[25] + x[25]*(F.dt*(K[K_e16]*x[45] + het[6]*x[12] + het[7]*x[18] + tj[J_hobr]) + T(1));
    R[29] = -F.dt*K[K_c7]*x[28]*x[47] - ck0[29] + x[29]*(F.dt*(K[K_c17a]*x[43] + K[K_c17b]*x[43] + tj[J_ch3o2h]) + T(1));
    R[31] = -ck0[31] + x[31]*(F.dt*(K[K_d91]*x[42] + tj[J_cfc12]) + T(1));
    R[34] = -ck0[34] + x[34]*(F.dt*(K[K_d94]*x[43] + tj[J_ch3ccl3]) + T(1));
    R[36] = -ck0[36] + x[36]*(F.dt*(K[K_d96]*x[42] + K[K_d97]*x[43] + tj[J_hcfc22]) + T(1));
    R[41] = -ck0[41] + x[41]*(F.dt*(K[K_e54]*x[43] + tj[J_ch2br2]) + T(1));
    R[42] = x[42];
    R[43] = x[43];
    R[49] = x[49];
    R[56] = x[56];
    const T N_t06_c0 = tj[J_hocl]*x[14];
    const T N_t06_c1 = K[K_d33]*x[47]*x[52];
    const bool sel_N_t06 = (N_t06_c0) <= (N_t06_c1);
    const T N_t06 = sel_N_t06 ? T(N_t06_c0) : T(N_t06_c1);
    const T N_t07_c0 = K[K_e5c]*x[52]*x[53];
    const T N_t07_c1 = tj[J_brcl]*x[26];
    const bool sel_N_t07 = (N_t07_c0) <= (N_t07_c1);
    const T N_t07 = sel_N_t07 ? T(N_t07_c0) : T(N_t07_c1);
    const T N_t09_c0 = K[K_e15]*x[47]*x[53];
    const T N_t09_c1 = tj[J_hobr]*x[25];
    const bool sel_N_t09 = (N_t09_c0) <= (N_t09_c1);
    const T N_t09 = sel_N_t09 ? T(N_t09_c0) : T(N_t09_c1);
    const T nr7_c0 = T(2)*x[45];
    const T nr7_c1 = nt_div<T>(T(2)*tj[J_no3_no], fmax(T(1e-30), tj[J_no3_no2] + tj[J_no3_no]));
    R[7] = -F.dt*(T(2)*F.o2*tj[J_o2] + K[K_a26]*x[47]*x[49] + K[K_c5]*x[28]*x[49]) + F.dt*(K[K_b3]*nr7_c0*x[48] + K[K_b9]*nr7_c1*x[46]*x[48] + K[K_d3]*nr7_c0*x[52] + nt_div<T>(T(2)*K[K_d60]*tj[J_cl2o2]*(x[52]*x[52]), F.hnm*K[K_d61] + tj[J_cl2o2]) + T(2)*K[K_hk1]*(x[45]*x[45]) + K[K_hk3]*nr7_c0*x[46] + N_t06 + T(2)*N_t07 + N_t09 + nr7_c1*tj[J_clono2_cl]*x[13] + x[45]*(K[K_a5]*x[43] + K[K_a7]*x[47]) + x[46]*(K[K_a2]*x[55] + K[K_a6]*x[43] + K[K_a6b]*x[47])) - ck0[7] + x[7];
}

// scaled Jacobian rows [0, 7, 12, 16, 19, 24, 34, 40, 41, 44, 48, 50, 54] (night equations) into their stored A slots
template <typename T, typename FF, typename PK, typename PJ>
__device__ __forceinline__ void nt_jacobian_night_w4_1(const FF& F, PK K, PK tj, PK het, const double* __restrict__ x, double floor_, PJ J) {
    const int fh = nt_exp_hi(floor_);
    const T xt0 = nt_cvt<T>(x[0]);
    const T xt1 = nt_cvt<T>(x[1]);
    const T xt2 = nt_cvt<T>(x[2]);
    const T xt3 = nt_cvt<T>(x[3]);
    const T xt4 = nt_cvt<T>(x[4]);
    const T xt5 = nt_cvt<T>(x[5]);
    const T xt6 = nt_cvt<T>(x[6]);
    const T xt7 = nt_cvt<T>(x[7]);
    const T xt8 = nt_cvt<T>(x[8]);
    const T xt9 = nt_cvt<T>(x[9]);
    const T xt10 = nt_cvt<T>(x[10]);
    const T xt11 = nt_cvt<T>(x[11]);
    const T xt12 = nt_cvt<T>(x[12]);
    const T xt13 = nt_cvt<T>(x[13]);
    const T xt14 = nt_cvt<T>(x[14]);
    const T xt15 = nt_cvt<T>(x[15]);
    const T xt16 = nt_cvt<T>(x[16]);
    const T xt17 = nt_cvt<T>(x[17]);
    const T xt18 = nt_cvt<T>(x[18]);
    const T xt19 = nt_cvt<T>(x[19]);
    const T xt20 = nt_cvt<T>(x[20]);
    const T xt21 = nt_cvt<T>(x[21]);
    const T xt22 = nt_cvt<T>(x[22]);
    const T xt23 = nt_cvt<T>(x[23]);
    const T xt24 = nt_cvt<T>(x[24]);
    const T xt25 = nt_cvt<T>(x[25]);
    const T xt26 = nt_cvt<T>(x[26]);
    const T xt27 = nt_cvt<T>(x[27]);
    const T xt28 = nt_cvt<T>(x[28]);
    const T xt29 = nt_cvt<T>(x[29]);
    const T xt30 = nt_cvt<T>(x[30]);
    const T xt31 = nt_cvt<T>(x[31]);
    const T xt32 = nt_cvt<T>(x[32]);
    const T xt33 = nt_cvt<T>(x[33]);
    const T xt34 = nt_cvt<T>(x[34]);
    const T xt35 = nt_cvt<T>(x[35]);
    const T xt36 = nt_cvt<T>(x[36]);
    const T xt37 = nt_cvt<T>(x[37]);
    const T xt38 = nt_cvt<T>(x[38]);
    const T xt39 = nt_cvt<T>(x[39]);
    const T xt40 = nt_cvt<T>(x[40]);
    const T xt41 = nt_cvt<T>(x[41]);
    const T xt42 = nt_cvt<T>(x[42]);
    const T xt43 = nt_cvt<T>(x[43]);
    const T xt44 = nt_cvt<T>(x[44]);
    const T xt45 = nt_cvt<T>(x[45]);
    const T xt46 = nt_cvt<T>(x[46]);
    const T xt47 = nt_cvt<T>(x[47]);
    const T xt48 = nt_cvt<T>(x[48]);
    const T xt49 = nt_cvt<T>(x[49]);
    const T xt50 = nt_cvt<T>(x[50]);
    const T xt51 = nt_cvt<T>(x[51]);
    const T xt52 = nt_cvt<T>(x[52]);
    const T xt53 = nt_cvt<T>(x[53]);
    const T xt54 = nt_cvt<T>(x[54]);
    const T xt55 = nt_cvt<T>(x[55]);
    const T xt56 = nt_cvt<T>(x[56]);
    const T cs0 = nt_scale<T>(nt_exp_hi(x[0]), fh);
    const T cs1 = nt_scale<T>(nt_exp_hi(x[1]), fh);
    const T cs2 = nt_scale<T>(nt_exp_hi(x[2]), fh);
    const T cs5 = nt_scale<T>(nt_exp_hi(x[5]), fh);
    const T cs12 = nt_scale<T>(nt_exp_hi(x[12]), fh);
    const T cs13 = nt_scale<T>(nt_exp_hi(x[13]), fh);
    const T cs14 = nt_scale<T>(nt_exp_hi(x[14]), fh);
    const T cs16 = nt_scale<T>(nt_exp_hi(x[16]), fh);
    const T cs18 = nt_scale<T>(nt_exp_hi(x[18]), fh);
    const T cs19 = nt_scale<T>(nt_exp_hi(x[19]), fh);
    const T cs20 = nt_scale<T>(nt_exp_hi(x[20]), fh);
    const T cs24 = nt_scale<T>(nt_exp_hi(x[24]), fh);
    const T cs25 = nt_scale<T>(nt_exp_hi(x[25]), fh);
    const T cs26 = nt_scale<T>(nt_exp_hi(x[26]), fh);
    const T cs27 = nt_scale<T>(nt_exp_hi(x[27]), fh);
    const T cs28 = nt_scale<T>(nt_exp_hi(x[28]), fh);
    const T cs34 = nt_scale<T>(nt_exp_hi(x[34]), fh);
    const T cs37 = nt_scale<T>(nt_exp_hi(x[37]), fh);
    const T cs38 = nt_scale<T>(nt_exp_hi(x[38]), fh);
    const T cs39 = nt_scale<T>(nt_exp_hi(x[39]), fh);
    const T cs41 = nt_scale<T>(nt_exp_hi(x[41]), fh);
    const T cs42 = nt_scale<T>(nt_exp_hi(x[42]), fh);
    const T cs43 = nt_scale<T>(nt_exp_hi(x[43]), fh);
    const T cs44 = nt_scale<T>(nt_exp_hi(x[44]), fh);
    const T cs45 = nt_scale<T>(nt_exp_hi(x[45]), fh);
    const T cs46 = nt_scale<T>(nt_exp_hi(x[46]), fh);
    const T cs47 = nt_scale<T>(nt_exp_hi(x[47]), fh);
    const T cs48 = nt_scale<T>(nt_exp_hi(x[48]), fh);
    const T cs49 = nt_scale<T>(nt_exp_hi(x[49]), fh);
    const T cs52 = nt_scale<T>(nt_exp_hi(x[52]), fh);
    const T cs53 = nt_scale<T>(nt_exp_hi(x[53]), fh);
    const T cs55 = nt_scale<T>(nt_exp_hi(x[55]), fh);
    {  // row 0
    const T rs0 = nt_rscale<T>(nt_exp_hi(x[0]), fh);
        const T nj0_c0 = K[K_b38] + K[K_b39];
        J[76] = (F.dt*(nj0_c0*xt42 + tj[J_n2o]) + T(1)) * (cs0 * rs0);
        J[77] = (F.dt*nj0_c0*xt0) * (cs42 * rs0);
    }
    {  // row 12
    const T rs12 = nt_rscale<T>(nt_exp_hi(x[12]), fh);
        const T nj12_c0 = F.dt*xt44;
        const T nj12_c1 = F.dt*xt12;
        const T nj12_c2 = F.dt*K[K_d9];
        J[250] = (-K[K_d5]*nj12_c0) * (cs1 * rs12);
        J[247] = (het[3]*nj12_c1) * (cs5 * rs12);
        J[253] = (F.dt*(F.parthcl*(K[K_d11]*xt43 + tj[J_hcl]) + F.rain_hcl + het[1]*xt13 + het[3]*xt5 + het[4]*xt14 + het[6]*xt25) + T(1)) * (cs12 * rs12);
        J[249] = (het[1]*nj12_c1) * (cs13 * rs12);
        J[251] = (het[4]*nj12_c1) * (cs14 * rs12);
        J[248] = (het[6]*nj12_c1) * (cs25 * rs12);
        J[252] = (-K[K_c10]*nj12_c0) * (cs27 * rs12);
        J[255] = (F.parthcl*K[K_d11]*nj12_c1 - nj12_c2*xt52) * (cs43 * rs12);
        J[254] = (-F.dt*(F.h2*K[K_d6] + K[K_c10]*xt27 + K[K_d5]*xt1 + K[K_d7]*xt47)) * (cs44 * rs12);
        J[256] = (-K[K_d7]*nj12_c0) * (cs47 * rs12);
        J[257] = (-nj12_c2*xt43) * (cs52 * rs12);
    }
    {  // row 16
    const T rs16 = nt_rscale<T>(nt_exp_hi(x[16]), fh);
        J[189] = (F.dt*(F.rain_h2o2 + K[K_a30]*xt43 + tj[J_h2o2]) + T(1)) * (cs16 * rs16);
        J[190] = (F.dt*K[K_a30]*xt16) * (cs43 * rs16);
        J[191] = (-T(2)*F.dt*K[K_a27]*xt47) * (cs47 * rs16);
    }
    {  // row 19
    const T rs19 = nt_rscale<T>(nt_exp_hi(x[19]), fh);
        const T nj19_c0 = F.dt*xt19;
        const T nj19_c1 = F.dt*K[K_e13];
        J[56] = (het[5]*nj19_c0) * (cs2 * rs19);
        J[55] = (F.dt*(K[K_e8]*xt45 + het[5]*xt2 + tj[J_brono2]) + T(1)) * (cs19 * rs19);
        J[58] = (K[K_e8]*nj19_c0) * (cs45 * rs19);
        J[57] = (-nj19_c1*xt53) * (cs48 * rs19);
        J[59] = (-nj19_c1*xt48) * (cs53 * rs19);
    }
    {  // row 24
    const T rs24 = nt_rscale<T>(nt_exp_hi(x[24]), fh);
        J[97] = (F.dt*(F.hnm*K[K_d61] + tj[J_cl2o2]) + T(1)) * (cs24 * rs24);
        J[98] = (-T(2)*F.dt*K[K_d60]*xt52) * (cs52 * rs24);
    }
    {  // row 34
    const T rs34 = nt_rscale<T>(nt_exp_hi(x[34]), fh);
        J[93] = (F.dt*(K[K_d94]*xt43 + tj[J_ch3ccl3]) + T(1)) * (cs34 * rs34);
        J[94] = (F.dt*K[K_d94]*xt34) * (cs43 * rs34);
    }
    {  // row 40
    const T rs40 = nt_rscale<T>(nt_exp_hi(x[40]), fh);
        const T nj40_c0 = T(2)*K[K_e54];
        J[16] = (F.dt*F.rain_hbr) * (cs18 * rs40);
        J[13] = (-F.dt*(K[K_e50]*xt42 + K[K_e51]*xt43 + tj[J_ch3br])) * (cs37 * rs40);
        J[11] = (-F.dt*(K[K_e52]*xt42 + tj[J_h1211])) * (cs38 * rs40);
        J[12] = (-F.dt*(K[K_e53]*xt42 + tj[J_h1301])) * (cs39 * rs40);
        J[15] = (-F.dt*(nj40_c0*xt43 + T(2)*tj[J_ch2br2])) * (cs41 * rs40);
        J[14] = (-F.dt*(K[K_e50]*xt37 + K[K_e52]*xt38 + K[K_e53]*xt39)) * (cs42 * rs40);
        J[17] = (-F.dt*(K[K_e51]*xt37 + nj40_c0*xt41)) * (cs43 * rs40);
    }
    {  // row 41
    const T rs41 = nt_rscale<T>(nt_exp_hi(x[41]), fh);
        J[125] = (F.dt*(K[K_e54]*xt43 + tj[J_ch2br2]) + T(1)) * (cs41 * rs41);
        J[126] = (F.dt*K[K_e54]*xt41) * (cs43 * rs41);
    }
    {  // row 44
    const T rs44 = nt_rscale<T>(nt_exp_hi(x[44]), fh);
        J[284] = T(0);
        J[288] = T(0);
        J[287] = T(0);
        J[285] = T(0);
        J[286] = T(0);
        J[292] = T(0);
        J[290] = T(0);
        J[294] = T(0);
        J[293] = T(0);
        J[289] = T(0);
        J[295] = T(0);
        J[296] = T(0);
        J[291] = T(0);
    }
    {  // row 50
    const T rs50 = nt_rscale<T>(nt_exp_hi(x[50]), fh);
        J[307] = T(0);
        J[311] = T(0);
        J[309] = T(0);
        J[313] = T(0);
        J[312] = T(0);
        J[308] = T(0);
        J[314] = T(0);
        J[315] = T(0);
        J[310] = T(0);
    }
    const T N_cno_c0 = nt_div<T>(K[K_b9], K[K_b12]);
    const T N_cno = N_cno_c0*xt46;
    const T d_N_cno_46 = N_cno_c0;
    const T N_dno = -N_cno + xt20;
    const T d_N_dno_20 = T(1);
    const T d_N_dno_46 = -d_N_cno_46;
    const T N_no2_c0 = N_cno + T(1e-30);
    const T N_no2_c1 = nt_div<T>(T(1e-30), N_no2_c0);
    const bool sel_N_no2 = (N_dno) > (T(1e-30));
    const T N_no2 = sel_N_no2 ? T(N_dno) : T(N_no2_c1*xt20);
    const T d_N_no2_20 = sel_N_no2 ? T(d_N_dno_20) : T(N_no2_c1);
    const T d_N_no2_46 = sel_N_no2 ? T(d_N_dno_46) : T(nt_div<T>(-T(1e-30)*d_N_cno_46*xt20, (N_no2_c0*N_no2_c0)));
    {  // row 48
    const T rs48 = nt_rscale<T>(nt_exp_hi(x[48]), fh);
        J[270] = (-d_N_no2_20) * (cs20 * rs48);
        J[269] = T(0);
        J[272] = T(0);
        J[275] = (-d_N_no2_46) * (cs46 * rs48);
        J[274] = T(0);
        J[271] = (T(1)) * (cs48 * rs48);
        J[276] = T(0);
        J[277] = T(0);
        J[273] = T(0);
    }
    const T N_no3_c0 = N_cno + T(1e-30);
    const T N_no3_c1 = nt_div<T>(T(1), N_no3_c0);
    const T N_no3_c2 = N_cno*N_no3_c1;
    const bool sel_N_no3 = (N_dno) > (T(1e-30));
    const T N_no3 = sel_N_no3 ? T(N_cno) : T(N_no3_c2*xt20);
    const T d_N_no3_20 = sel_N_no3 ? T(T(0)) : T(N_no3_c2);
    const T d_N_no3_46 = sel_N_no3 ? T(d_N_cno_46) : T(d_N_cno_46*(nt_div<T>(-N_cno*xt20, (N_no3_c0*N_no3_c0)) + N_no3_c1*xt20));
    {  // row 54
    const T rs54 = nt_rscale<T>(nt_exp_hi(x[54]), fh);
        J[68] = (-d_N_no3_20) * (cs20 * rs54);
        J[70] = (-d_N_no3_46) * (cs46 * rs54);
        J[69] = T(0);
    }
    const T N_t06_c0 = tj[J_hocl]*xt14;
    const T N_t06_c1 = K[K_d33]*xt52;
    const T N_t06_c2 = N_t06_c1*xt47;
    const bool sel_N_t06 = (N_t06_c0) <= (N_t06_c2);
    const T N_t06 = sel_N_t06 ? T(N_t06_c0) : T(N_t06_c2);
    const T d_N_t06_14 = sel_N_t06 ? T(tj[J_hocl]) : T(T(0));
    const T d_N_t06_47 = sel_N_t06 ? T(T(0)) : T(N_t06_c1);
    const T d_N_t06_52 = sel_N_t06 ? T(T(0)) : T(K[K_d33]*xt47);
    const T N_t07_c0 = K[K_e5c]*xt53;
    const T N_t07_c1 = N_t07_c0*xt52;
    const T N_t07_c2 = tj[J_brcl]*xt26;
    const bool sel_N_t07 = (N_t07_c1) <= (N_t07_c2);
    const T N_t07 = sel_N_t07 ? T(N_t07_c1) : T(N_t07_c2);
    const T d_N_t07_26 = sel_N_t07 ? T(T(0)) : T(tj[J_brcl]);
    const T d_N_t07_52 = sel_N_t07 ? T(N_t07_c0) : T(T(0));
    const T d_N_t07_53 = sel_N_t07 ? T(K[K_e5c]*xt52) : T(T(0));
    const T N_t09_c0 = K[K_e15]*xt53;
    const T N_t09_c1 = N_t09_c0*xt47;
    const T N_t09_c2 = tj[J_hobr]*xt25;
    const bool sel_N_t09 = (N_t09_c1) <= (N_t09_c2);
    const T N_t09 = sel_N_t09 ? T(N_t09_c1) : T(N_t09_c2);
    const T d_N_t09_25 = sel_N_t09 ? T(T(0)) : T(tj[J_hobr]);
    const T d_N_t09_47 = sel_N_t09 ? T(N_t09_c0) : T(T(0));
    const T d_N_t09_53 = sel_N_t09 ? T(K[K_e15]*xt47) : T(T(0));
    {  // row 7
    const T rs7 = nt_rscale<T>(nt_exp_hi(x[7]), fh);
        const T nj7_c0 = T(2)*F.dt;
        const T nj7_c1 = nt_div<T>(tj[J_no3_no], fmax(T(1e-30), tj[J_no3_no2] + tj[J_no3_no]));
        const T nj7_c2 = F.dt*xt49;
        const T nj7_c3 = T(2)*K[K_b3];
        const T nj7_c4 = T(2)*K[K_d3];
        const T nj7_c5 = T(2)*K[K_hk3];
        const T nj7_c6 = T(2)*K[K_b9]*nj7_c1;
        J[105] = (nj7_c0*nj7_c1*tj[J_clono2_cl]) * (cs13 * rs7);
        J[106] = (F.dt*d_N_t06_14) * (cs14 * rs7);
        J[104] = (F.dt*d_N_t09_25) * (cs25 * rs7);
        J[103] = (d_N_t07_26*nj7_c0) * (cs26 * rs7);
        J[108] = (-K[K_c5]*nj7_c2) * (cs28 * rs7);
        J[112] = (F.dt*(K[K_a5]*xt45 + K[K_a6]*xt46)) * (cs43 * rs7);
        J[110] = (F.dt*(K[K_a5]*xt43 + K[K_a7]*xt47 + T(4)*K[K_hk1]*xt45 + nj7_c3*xt48 + nj7_c4*xt52 + nj7_c5*xt46)) * (cs45 * rs7);
        J[114] = (F.dt*(K[K_a2]*xt55 + K[K_a6]*xt43 + K[K_a6b]*xt47 + nj7_c5*xt45 + nj7_c6*xt48)) * (cs46 * rs7);
        J[113] = (F.dt*d_N_t06_47 + F.dt*d_N_t09_47 + F.dt*(K[K_a6b]*xt46 + K[K_a7]*xt45) - K[K_a26]*nj7_c2) * (cs47 * rs7);
        J[109] = (F.dt*(nj7_c3*xt45 + nj7_c6*xt46)) * (cs48 * rs7);
        J[115] = (-F.dt*(K[K_a26]*xt47 + K[K_c5]*xt28)) * (cs49 * rs7);
        J[116] = (F.dt*d_N_t06_52 + F.dt*(nt_div<T>(T(4)*K[K_d60]*tj[J_cl2o2]*xt52, F.hnm*K[K_d61] + tj[J_cl2o2]) + nj7_c4*xt45) + d_N_t07_52*nj7_c0) * (cs52 * rs7);
        J[111] = (F.dt*d_N_t09_53 + d_N_t07_53*nj7_c0) * (cs53 * rs7);
        J[107] = (F.dt*K[K_a2]*xt46) * (cs55 * rs7);
    }
}

// residual rows [0, 10, 13, 16, 19, 20, 23, 28, 35, 40, 44, 48, 50, 52, 53] (night equations, FP64)
template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>
__device__ __forceinline__ void nt_residual_night_w4_2(const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {
    R[0] = -ck0[0] + x[0]*(F.dt*(tj[J_n2o] + x[42]*(K[K_b38] + K[K_b39])) + T(1));
    R[10] = -ck0[10] + x[10];
    R[13] = -F.dt*K[K_d31]*x[48]*x[52] - ck0[13] + x[13]*(F.dt*(K[K_d32]*x[45] + het[0]*x[2] + het[1]*x[12] + tj[J_clono2_cl] + tj[J_clono2_clo]) + T(1));
    R[16] = -F.dt*K[K_a27]*(x[47]*x[47]) - ck0[16] + x[16]*(F.dt*(F.rain_h2o2 + K[K_a30]*x[43] + tj[J_h2o2]) + T(1));
    R[19] = -F.dt*K[K_e13]*x[48]*x[53] - ck0[19] + x[19]*(F.dt*(K[K_e8]*x[45] + het[5]*x[2] + tj[J_brono2]) + T(1));
    const T nr20_c0 = F.parthno3*x[4];
    R[20] = F.dt*(T(2)*K[K_b6]*x[49]*x[51] + x[48]*(T(2)*K[K_b12]*x[54] + K[K_b22]*x[43] + K[K_b23]*x[47] + K[K_d31]*x[52] + K[K_d36]*x[44] + K[K_e13]*x[53])) - F.dt*(K[K_b27]*nr20_c0*x[43] + T(2)*K[K_b39]*x[0]*x[42] + K[K_d32]*x[13]*x[45] + K[K_e8]*x[19]*x[45] + nr20_c0*tj[J_hno3] + tj[J_brono2]*x[19] + tj[J_clno2]*x[17] + x[13]*(tj[J_clono2_cl] + tj[J_clono2_clo]) + x[21]*(F.hnm*K[K_b24] + K[K_b28]*x[43] + tj[J_hno4]) + x[5]*(T(2)*F.hnm*K[K_b32] + T(2)*tj[J_n2o5])) - ck0[20] + x[20];
    R[23] = F.dt*(K[K_c19]*x[27]*x[50] + K[K_e7]*x[47]*x[50] + x[53]*(K[K_e13]*x[48] + K[K_e15]*x[47] + K[K_e5c]*x[52])) - F.dt*(F.parthbr*x[18]*(K[K_e11]*x[43] + K[K_e9]*x[42] + tj[J_hbr]) + K[K_e16]*x[25]*x[45] + K[K_e8]*x[19]*x[45] + T(2)*het[7]*x[18]*x[25] + tj[J_brcl]*x[26] + tj[J_brono2]*x[19] + tj[J_hobr]*x[25]) - ck0[23] + x[23];
    R[28] = -F.dt*(F.o2*K[K_c4]*x[56] + K[K_c17a]*x[29]*x[43]) - ck0[28] + x[28]*(F.dt*(T(2)*K[K_c14]*x[28] + K[K_c18]*x[52] + K[K_c5]*x[49] + K[K_c7]*x[47]) + T(1));
    R[35] = -ck0[35] + x[35]*(F.dt*(K[K_d95]*x[43] + tj[J_ch3cl]) + T(1));
    R[40] = F.dt*F.rain_hbr*x[18] - F.dt*(x[37]*(K[K_e50]*x[42] + K[K_e51]*x[43] + tj[J_ch3br]) + x[38]*(K[K_e52]*x[42] + tj[J_h1211]) + x[39]*(K[K_e53]*x[42] + tj[J_h1301]) + x[41]*(T(2)*K[K_e54]*x[43] + T(2)*tj[J_ch2br2])) - ck0[40] + x[40];
    R[44] = x[44];
    R[50] = x[50];
    const T N_cno = nt_div<T>(K[K_b9]*x[46], K[K_b12]);
    const T N_dno = -N_cno + x[20];
    const bool sel_N_no2 = (N_dno) > (T(1e-30));
    const T N_no2 = sel_N_no2 ? T(N_dno) : T(nt_div<T>(T(1e-30)*x[20], N_cno + T(1e-30)));
    R[48] = -N_no2 + x[48];
    const bool sel_N_clo = (x[22]) >= (T(0));
    const T N_clo = sel_N_clo ? T(x[22]) : T(T(0));
    R[52] = -N_clo + x[52];
    const bool sel_N_bro = (x[23]) >= (T(0));
    const T N_bro = sel_N_bro ? T(x[23]) : T(T(0));
    R[53] = -N_bro + x[53];
}

// scaled Jacobian rows [5, 8, 13, 17, 18, 20, 23, 27, 33, 36, 39, 42, 45, 51] (night equations) into their stored A slots
template <typename T, typename FF, typename PK, typename PJ>
__device__ __forceinline__ void nt_jacobian_night_w4_2(const FF& F, PK K, PK tj, PK het, const double* __restrict__ x, double floor_, PJ J) {
    const int fh = nt_exp_hi(floor_);
    const T xt0 = nt_cvt<T>(x[0]);
    const T xt1 = nt_cvt<T>(x[1]);
    const T xt2 = nt_cvt<T>(x[2]);
    const T xt3 = nt_cvt<T>(x[3]);
    const T xt4 = nt_cvt<T>(x[4]);
    const T xt5 = nt_cvt<T>(x[5]);
    const T xt6 = nt_cvt<T>(x[6]);
    const T xt7 = nt_cvt<T>(x[7]);
    const T xt8 = nt_cvt<T>(x[8]);
    const T xt9 = nt_cvt<T>(x[9]);
    const T xt10 = nt_cvt<T>(x[10]);
    const T xt11 = nt_cvt<T>(x[11]);
    const T xt12 = nt_cvt<T>(x[12]);
    const T xt13 = nt_cvt<T>(x[13]);
    const T xt14 = nt_cvt<T>(x[14]);
    const T xt15 = nt_cvt<T>(x[15]);
    const T xt16 = nt_cvt<T>(x[16]);
    const T xt17 = nt_cvt<T>(x[17]);
    const T xt18 = nt_cvt<T>(x[18]);
    const T xt19 = nt_cvt<T>(x[19]);
    const T xt20 = nt_cvt<T>(x[20]);
    const T xt21 = nt_cvt<T>(x[21]);
    const T xt22 = nt_cvt<T>(x[22]);
    const T xt23 = nt_cvt<T>(x[23]);
    const T xt24 = nt_cvt<T>(x[24]);
    const T xt25 = nt_cvt<T>(x[25]);
    const T xt26 = nt_cvt<T>(x[26]);
    const T xt27 = nt_cvt<T>(x[27]);
    const T xt28 = nt_cvt<T>(x[28]);
    const T xt29 = nt_cvt<T>(x[29]);
    const T xt30 = nt_cvt<T>(x[30]);
    const T xt31 = nt_cvt<T>(x[31]);
    const T xt32 = nt_cvt<T>(x[32]);
    const T xt33 = nt_cvt<T>(x[33]);
    const T xt34 = nt_cvt<T>(x[34]);
    const T xt35 = nt_cvt<T>(x[35]);
    const T xt36 = nt_cvt<T>(x[36]);
    const T xt37 = nt_cvt<T>(x[37]);
    const T xt38 = nt_cvt<T>(x[38]);
    const T xt39 = nt_cvt<T>(x[39]);
    const T xt40 = nt_cvt<T>(x[40]);
    const T xt41 = nt_cvt<T>(x[41]);
    const T xt42 = nt_cvt<T>(x[42]);
    const T xt43 = nt_cvt<T>(x[43]);
    const T xt44 = nt_cvt<T>(x[44]);
    const T xt45 = nt_cvt<T>(x[45]);
    const T xt46 = nt_cvt<T>(x[46]);
    const T xt47 = nt_cvt<T>(x[47]);
    const T xt48 = nt_cvt<T>(x[48]);
    const T xt49 = nt_cvt<T>(x[49]);
    const T xt50 = nt_cvt<T>(x[50]);
    const T xt51 = nt_cvt<T>(x[51]);
    const T xt52 = nt_cvt<T>(x[52]);
    const T xt53 = nt_cvt<T>(x[53]);
    const T xt54 = nt_cvt<T>(x[54]);
    const T xt55 = nt_cvt<T>(x[55]);
    const T xt56 = nt_cvt<T>(x[56]);
    const T cs0 = nt_scale<T>(nt_exp_hi(x[0]), fh);
    const T cs1 = nt_scale<T>(nt_exp_hi(x[1]), fh);
    const T cs2 = nt_scale<T>(nt_exp_hi(x[2]), fh);
    const T cs4 = nt_scale<T>(nt_exp_hi(x[4]), fh);
    const T cs5 = nt_scale<T>(nt_exp_hi(x[5]), fh);
    const T cs8 = nt_scale<T>(nt_exp_hi(x[8]), fh);
    const T cs12 = nt_scale<T>(nt_exp_hi(x[12]), fh);
    const T cs13 = nt_scale<T>(nt_exp_hi(x[13]), fh);
    const T cs14 = nt_scale<T>(nt_exp_hi(x[14]), fh);
    const T cs17 = nt_scale<T>(nt_exp_hi(x[17]), fh);
    const T cs18 = nt_scale<T>(nt_exp_hi(x[18]), fh);
    const T cs19 = nt_scale<T>(nt_exp_hi(x[19]), fh);
    const T cs21 = nt_scale<T>(nt_exp_hi(x[21]), fh);
    const T cs25 = nt_scale<T>(nt_exp_hi(x[25]), fh);
    const T cs26 = nt_scale<T>(nt_exp_hi(x[26]), fh);
    const T cs27 = nt_scale<T>(nt_exp_hi(x[27]), fh);
    const T cs28 = nt_scale<T>(nt_exp_hi(x[28]), fh);
    const T cs29 = nt_scale<T>(nt_exp_hi(x[29]), fh);
    const T cs33 = nt_scale<T>(nt_exp_hi(x[33]), fh);
    const T cs36 = nt_scale<T>(nt_exp_hi(x[36]), fh);
    const T cs39 = nt_scale<T>(nt_exp_hi(x[39]), fh);
    const T cs42 = nt_scale<T>(nt_exp_hi(x[42]), fh);
    const T cs43 = nt_scale<T>(nt_exp_hi(x[43]), fh);
    const T cs44 = nt_scale<T>(nt_exp_hi(x[44]), fh);
    const T cs45 = nt_scale<T>(nt_exp_hi(x[45]), fh);
    const T cs46 = nt_scale<T>(nt_exp_hi(x[46]), fh);
    const T cs47 = nt_scale<T>(nt_exp_hi(x[47]), fh);
    const T cs48 = nt_scale<T>(nt_exp_hi(x[48]), fh);
    const T cs49 = nt_scale<T>(nt_exp_hi(x[49]), fh);
    const T cs50 = nt_scale<T>(nt_exp_hi(x[50]), fh);
    const T cs51 = nt_scale<T>(nt_exp_hi(x[51]), fh);
    const T cs52 = nt_scale<T>(nt_exp_hi(x[52]), fh);
    const T cs53 = nt_scale<T>(nt_exp_hi(x[53]), fh);
    const T cs54 = nt_scale<T>(nt_exp_hi(x[54]), fh);
    const T cs55 = nt_scale<T>(nt_exp_hi(x[55]), fh);
    const T cs56 = nt_scale<T>(nt_exp_hi(x[56]), fh);
    {  // row 5
    const T rs5 = nt_rscale<T>(nt_exp_hi(x[5]), fh);
        const T nj5_c0 = F.dt*xt5;
        const T nj5_c1 = F.dt*K[K_b12];
        J[74] = (het[2]*nj5_c0) * (cs2 * rs5);
        J[72] = (F.dt*(F.hnm*K[K_b32] + het[2]*xt2 + het[3]*xt12 + tj[J_n2o5]) + T(1)) * (cs5 * rs5);
        J[73] = (het[3]*nj5_c0) * (cs12 * rs5);
        J[75] = (-nj5_c1*xt54) * (cs48 * rs5);
        J[71] = (-nj5_c1*xt48) * (cs54 * rs5);
    }
    {  // row 8
    const T rs8 = nt_rscale<T>(nt_exp_hi(x[8]), fh);
        const T nj8_c0 = F.dt*K[K_a36];
        J[160] = (nj8_c0*xt43 + T(1)) * (cs8 * rs8);
        J[161] = (-F.dt*tj[J_ch2o_co]) * (cs27 * rs8);
        J[165] = (nj8_c0*xt8) * (cs43 * rs8);
        J[163] = T(0);
        J[162] = T(0);
        J[164] = T(0);
    }
    {  // row 13
    const T rs13 = nt_rscale<T>(nt_exp_hi(x[13]), fh);
        const T nj13_c0 = F.dt*xt13;
        const T nj13_c1 = F.dt*K[K_d31];
        J[89] = (het[0]*nj13_c0) * (cs2 * rs13);
        J[88] = (het[1]*nj13_c0) * (cs12 * rs13);
        J[87] = (F.dt*(K[K_d32]*xt45 + het[0]*xt2 + het[1]*xt12 + tj[J_clono2_cl] + tj[J_clono2_clo]) + T(1)) * (cs13 * rs13);
        J[91] = (K[K_d32]*nj13_c0) * (cs45 * rs13);
        J[90] = (-nj13_c1*xt52) * (cs48 * rs13);
        J[92] = (-nj13_c1*xt48) * (cs52 * rs13);
    }
    {  // row 17
    const T rs17 = nt_rscale<T>(nt_exp_hi(x[17]), fh);
        const T nj17_c0 = F.dt*het[3];
        const T nj17_c1 = F.dt*K[K_d36];
        J[26] = (-nj17_c0*xt12) * (cs5 * rs17);
        J[27] = (-nj17_c0*xt5) * (cs12 * rs17);
        J[25] = (F.dt*tj[J_clno2] + T(1)) * (cs17 * rs17);
        J[29] = (-nj17_c1*xt48) * (cs44 * rs17);
        J[28] = (-nj17_c1*xt44) * (cs48 * rs17);
    }
    {  // row 18
    const T rs18 = nt_rscale<T>(nt_exp_hi(x[18]), fh);
        const T nj18_c0 = F.dt*xt18;
        const T nj18_c1 = F.dt*xt50;
        const T nj18_c2 = F.parthbr*nj18_c0;
        J[183] = (het[8]*nj18_c0) * (cs14 * rs18);
        J[184] = (F.dt*(F.parthbr*(K[K_e11]*xt43 + K[K_e9]*xt42 + tj[J_hbr]) + F.rain_hbr + het[7]*xt25 + het[8]*xt14) + T(1)) * (cs18 * rs18);
        J[181] = (het[7]*nj18_c0) * (cs25 * rs18);
        J[185] = (-K[K_c19]*nj18_c1) * (cs27 * rs18);
        J[182] = (K[K_e9]*nj18_c2) * (cs42 * rs18);
        J[187] = (K[K_e11]*nj18_c2) * (cs43 * rs18);
        J[188] = (-K[K_e7]*nj18_c1) * (cs47 * rs18);
        J[186] = (-F.dt*(K[K_c19]*xt27 + K[K_e7]*xt47)) * (cs50 * rs18);
    }
    {  // row 20
    const T rs20 = nt_rscale<T>(nt_exp_hi(x[20]), fh);
        const T nj20_c0 = T(2)*F.dt;
        const T nj20_c1 = K[K_b39]*nj20_c0;
        const T nj20_c2 = F.parthno3*K[K_b27];
        const T nj20_c3 = F.dt*xt48;
        const T nj20_c4 = T(2)*K[K_b12];
        const T nj20_c5 = K[K_b6]*nj20_c0;
        J[233] = (-nj20_c1*xt42) * (cs0 * rs20);
        J[237] = (-F.dt*(F.parthno3*tj[J_hno3] + nj20_c2*xt43)) * (cs4 * rs20);
        J[232] = (-F.dt*(T(2)*F.hnm*K[K_b32] + T(2)*tj[J_n2o5])) * (cs5 * rs20);
        J[235] = (-F.dt*(K[K_d32]*xt45 + tj[J_clono2_cl] + tj[J_clono2_clo])) * (cs13 * rs20);
        J[229] = (-F.dt*tj[J_clno2]) * (cs17 * rs20);
        J[230] = (-F.dt*(K[K_e8]*xt45 + tj[J_brono2])) * (cs19 * rs20);
        J[238] = (-F.dt*(F.hnm*K[K_b24] + K[K_b28]*xt43 + tj[J_hno4])) * (cs21 * rs20);
        J[236] = (-nj20_c1*xt0) * (cs42 * rs20);
        J[243] = (-F.dt*(K[K_b28]*xt21 + nj20_c2*xt4) + K[K_b22]*nj20_c3) * (cs43 * rs20);
        J[241] = (K[K_d36]*nj20_c3) * (cs44 * rs20);
        J[240] = (-F.dt*(K[K_d32]*xt13 + K[K_e8]*xt19)) * (cs45 * rs20);
        J[244] = (K[K_b23]*nj20_c3) * (cs47 * rs20);
        J[239] = (F.dt*(K[K_b22]*xt43 + K[K_b23]*xt47 + K[K_d31]*xt52 + K[K_d36]*xt44 + K[K_e13]*xt53 + nj20_c4*xt54)) * (cs48 * rs20);
        J[245] = (nj20_c5*xt51) * (cs49 * rs20);
        J[234] = (nj20_c5*xt49) * (cs51 * rs20);
        J[246] = (K[K_d31]*nj20_c3) * (cs52 * rs20);
        J[242] = (K[K_e13]*nj20_c3) * (cs53 * rs20);
        J[231] = (nj20_c3*nj20_c4) * (cs54 * rs20);
    }
    {  // row 23
    const T rs23 = nt_rscale<T>(nt_exp_hi(x[23]), fh);
        const T nj23_c0 = T(2)*het[7];
        const T nj23_c1 = F.dt*F.parthbr*xt18;
        const T nj23_c2 = F.dt*xt53;
        J[196] = (-F.dt*(F.parthbr*(K[K_e11]*xt43 + K[K_e9]*xt42 + tj[J_hbr]) + nj23_c0*xt25)) * (cs18 * rs23);
        J[193] = (-F.dt*(K[K_e8]*xt45 + tj[J_brono2])) * (cs19 * rs23);
        J[194] = (-F.dt*(K[K_e16]*xt45 + nj23_c0*xt18 + tj[J_hobr])) * (cs25 * rs23);
        J[192] = (-F.dt*tj[J_brcl]) * (cs26 * rs23);
        J[197] = (F.dt*K[K_c19]*xt50) * (cs27 * rs23);
        J[195] = (-K[K_e9]*nj23_c1) * (cs42 * rs23);
        J[202] = (-K[K_e11]*nj23_c1) * (cs43 * rs23);
        J[199] = (-F.dt*(K[K_e16]*xt25 + K[K_e8]*xt19)) * (cs45 * rs23);
        J[203] = (F.dt*(K[K_e15]*xt53 + K[K_e7]*xt50)) * (cs47 * rs23);
        J[198] = (K[K_e13]*nj23_c2) * (cs48 * rs23);
        J[201] = (F.dt*(K[K_c19]*xt27 + K[K_e7]*xt47)) * (cs50 * rs23);
        J[204] = (K[K_e5c]*nj23_c2) * (cs52 * rs23);
        J[200] = (F.dt*(K[K_e13]*xt48 + K[K_e15]*xt47 + K[K_e5c]*xt52)) * (cs53 * rs23);
    }
    {  // row 27
    const T rs27 = nt_rscale<T>(nt_exp_hi(x[27]), fh);
        const T nj27_c0 = F.dt*K[K_c1c];
        const T nj27_c1 = F.dt*K[K_c17b];
        const T nj27_c2 = F.dt*xt27;
        const T nj27_c3 = F.dt*K[K_c3];
        J[219] = (-nj27_c0*xt42) * (cs1 * rs27);
        J[222] = (F.dt*(K[K_c10]*xt44 + K[K_c19]*xt50 + K[K_c8]*xt43 + K[K_c9]*xt45 + tj[J_ch2o_co] + tj[J_ch2o_hco]) + T(1)) * (cs27 * rs27);
        J[221] = T(0);
        J[217] = (-nj27_c1*xt43) * (cs29 * rs27);
        J[218] = (-nj27_c0*xt1) * (cs42 * rs27);
        J[226] = (F.dt*K[K_c8]*xt27 - nj27_c1*xt29) * (cs43 * rs27);
        J[224] = (K[K_c10]*nj27_c2) * (cs44 * rs27);
        J[223] = (F.dt*K[K_c9]*xt27 - nj27_c3*xt56) * (cs45 * rs27);
        J[227] = T(0);
        J[225] = (K[K_c19]*nj27_c2) * (cs50 * rs27);
        J[228] = T(0);
        J[220] = (-nj27_c3*xt45) * (cs56 * rs27);
    }
    {  // row 33
    const T rs33 = nt_rscale<T>(nt_exp_hi(x[33]), fh);
        J[32] = (F.dt*(K[K_d93]*xt42 + tj[J_ccl4]) + T(1)) * (cs33 * rs33);
        J[33] = (F.dt*K[K_d93]*xt33) * (cs42 * rs33);
    }
    {  // row 36
    const T rs36 = nt_rscale<T>(nt_exp_hi(x[36]), fh);
        const T nj36_c0 = F.dt*xt36;
        J[38] = (F.dt*(K[K_d96]*xt42 + K[K_d97]*xt43 + tj[J_hcfc22]) + T(1)) * (cs36 * rs36);
        J[39] = (K[K_d96]*nj36_c0) * (cs42 * rs36);
        J[40] = (K[K_d97]*nj36_c0) * (cs43 * rs36);
    }
    {  // row 39
    const T rs39 = nt_rscale<T>(nt_exp_hi(x[39]), fh);
        J[50] = (F.dt*(K[K_e53]*xt42 + tj[J_h1301]) + T(1)) * (cs39 * rs39);
        J[51] = (F.dt*K[K_e53]*xt39) * (cs42 * rs39);
    }
    {  // row 42
    const T rs42 = nt_rscale<T>(nt_exp_hi(x[42]), fh);
        J[99] = T(0);
    }
    {  // row 45
    const T rs45 = nt_rscale<T>(nt_exp_hi(x[45]), fh);
        J[280] = T(0);
        J[279] = T(0);
        J[282] = T(0);
        J[281] = T(0);
        J[283] = T(0);
        J[278] = T(0);
    }
    {  // row 51
    const T rs51 = nt_rscale<T>(nt_exp_hi(x[51]), fh);
        J[78] = T(0);
    }
}

// residual rows [2, 3, 4, 5, 6, 11, 17, 18, 30, 32, 38, 45, 51, 54] (night equations, FP64)
template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>
__device__ __forceinline__ void nt_residual_night_w4_3(const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {
    const T nr2_c0 = x[29]*x[43];
    R[2] = -F.dt*(F.h2*K[K_a19]*x[43] + F.parthcl*K[K_d11]*x[12]*x[43] + F.parthno3*K[K_b27]*x[43]*x[4] + K[K_a30]*x[16]*x[43] + K[K_a31]*(x[43]*x[43]) + K[K_c17a]*nr2_c0 + K[K_c17b]*nr2_c0 + K[K_c2]*x[1]*x[43] + K[K_c8]*x[27]*x[43] + x[47]*(K[K_a17]*x[43] + T(1.6e-12)*x[55])) - ck0[2] + x[2]*(F.dt*F.parth2o*(K[K_a1et]*x[42] + tj[J_h2o]) + T(1));
    R[3] = -T(2)*F.dt*K[K_b39]*x[0]*x[42] + F.dt*(F.rain_hno3*x[4] + T(2)*K[K_b6]*x[49]*x[51]) - ck0[3] + x[3];
    R[4] = -F.dt*(K[K_b22]*x[43]*x[48] + het[0]*x[13]*x[2] + het[1]*x[12]*x[13] + T(2)*het[2]*x[2]*x[5] + het[3]*x[12]*x[5] + het[5]*x[19]*x[2]) - ck0[4] + x[4]*(F.dt*(F.parthno3*(K[K_b27]*x[43] + tj[J_hno3]) + F.rain_hno3) + T(1));
    R[5] = -F.dt*K[K_b12]*x[48]*x[54] - ck0[5] + x[5]*(F.dt*(F.hnm*K[K_b32] + het[2]*x[2] + het[3]*x[12] + tj[J_n2o5]) + T(1));
    const T nr6_c0 = T(3)*x[42];
    R[6] = F.dt*F.rain_hcl*x[12] - F.dt*(x[30]*(K[K_d90]*nr6_c0 + T(3)*tj[J_cfc11]) + x[31]*(T(2)*K[K_d91]*x[42] + T(2)*tj[J_cfc12]) + x[32]*(K[K_d92]*nr6_c0 + T(3)*tj[J_cfc113]) + x[33]*(T(4)*K[K_d93]*x[42] + T(4)*tj[J_ccl4]) + x[34]*(T(3)*K[K_d94]*x[43] + T(3)*tj[J_ch3ccl3]) + x[35]*(K[K_d95]*x[43] + tj[J_ch3cl]) + x[36]*(K[K_d96]*x[42] + K[K_d97]*x[43] + tj[J_hcfc22]) + x[38]*(K[K_e52]*x[42] + tj[J_h1211])) - ck0[6] + x[6];
    R[11] = -ck0[11] + x[11];
    R[17] = -F.dt*(K[K_d36]*x[44]*x[48] + het[3]*x[12]*x[5]) - ck0[17] + x[17]*(F.dt*tj[J_clno2] + T(1));
    R[18] = -F.dt*(K[K_c19]*x[27]*x[50] + K[K_e7]*x[47]*x[50]) - ck0[18] + x[18]*(F.dt*(F.parthbr*(K[K_e11]*x[43] + K[K_e9]*x[42] + tj[J_hbr]) + F.rain_hbr + het[7]*x[25] + het[8]*x[14]) + T(1));
    R[30] = -ck0[30] + x[30]*(F.dt*(K[K_d90]*x[42] + tj[J_cfc11]) + T(1));
    R[32] = -ck0[32] + x[32]*(F.dt*(K[K_d92]*x[42] + tj[J_cfc113]) + T(1));
    R[38] = -ck0[38] + x[38]*(F.dt*(K[K_e52]*x[42] + tj[J_h1211]) + T(1));
    R[45] = x[45];
    R[51] = x[51];
    const T N_cno = nt_div<T>(K[K_b9]*x[46], K[K_b12]);
    const T N_dno = -N_cno + x[20];
    const bool sel_N_no3 = (N_dno) > (T(1e-30));
    const T N_no3 = sel_N_no3 ? T(N_cno) : T(nt_div<T>(N_cno*x[20], N_cno + T(1e-30)));
    R[54] = -N_no3 + x[54];
}

// scaled Jacobian rows [1, 2, 4, 6, 15, 28, 29, 30, 32, 37, 38, 46, 47, 55] (night equations) into their stored A slots
template <typename T, typename FF, typename PK, typename PJ>
__device__ __forceinline__ void nt_jacobian_night_w4_3(const FF& F, PK K, PK tj, PK het, const double* __restrict__ x, double floor_, PJ J) {
    const int fh = nt_exp_hi(floor_);
    const T xt0 = nt_cvt<T>(x[0]);
    const T xt1 = nt_cvt<T>(x[1]);
    const T xt2 = nt_cvt<T>(x[2]);
    const T xt3 = nt_cvt<T>(x[3]);
    const T xt4 = nt_cvt<T>(x[4]);
    const T xt5 = nt_cvt<T>(x[5]);
    const T xt6 = nt_cvt<T>(x[6]);
    const T xt7 = nt_cvt<T>(x[7]);
    const T xt8 = nt_cvt<T>(x[8]);
    const T xt9 = nt_cvt<T>(x[9]);
    const T xt10 = nt_cvt<T>(x[10]);
    const T xt11 = nt_cvt<T>(x[11]);
    const T xt12 = nt_cvt<T>(x[12]);
    const T xt13 = nt_cvt<T>(x[13]);
    const T xt14 = nt_cvt<T>(x[14]);
    const T xt15 = nt_cvt<T>(x[15]);
    const T xt16 = nt_cvt<T>(x[16]);
    const T xt17 = nt_cvt<T>(x[17]);
    const T xt18 = nt_cvt<T>(x[18]);
    const T xt19 = nt_cvt<T>(x[19]);
    const T xt20 = nt_cvt<T>(x[20]);
    const T xt21 = nt_cvt<T>(x[21]);
    const T xt22 = nt_cvt<T>(x[22]);
    const T xt23 = nt_cvt<T>(x[23]);
    const T xt24 = nt_cvt<T>(x[24]);
    const T xt25 = nt_cvt<T>(x[25]);
    const T xt26 = nt_cvt<T>(x[26]);
    const T xt27 = nt_cvt<T>(x[27]);
    const T xt28 = nt_cvt<T>(x[28]);
    const T xt29 = nt_cvt<T>(x[29]);
    const T xt30 = nt_cvt<T>(x[30]);
    const T xt31 = nt_cvt<T>(x[31]);
    const T xt32 = nt_cvt<T>(x[32]);
    const T xt33 = nt_cvt<T>(x[33]);
    const T xt34 = nt_cvt<T>(x[34]);
    const T xt35 = nt_cvt<T>(x[35]);
    const T xt36 = nt_cvt<T>(x[36]);
    const T xt37 = nt_cvt<T>(x[37]);
    const T xt38 = nt_cvt<T>(x[38]);
    const T xt39 = nt_cvt<T>(x[39]);
    const T xt40 = nt_cvt<T>(x[40]);
    const T xt41 = nt_cvt<T>(x[41]);
    const T xt42 = nt_cvt<T>(x[42]);
    const T xt43 = nt_cvt<T>(x[43]);
    const T xt44 = nt_cvt<T>(x[44]);
    const T xt45 = nt_cvt<T>(x[45]);
    const T xt46 = nt_cvt<T>(x[46]);
    const T xt47 = nt_cvt<T>(x[47]);
    const T xt48 = nt_cvt<T>(x[48]);
    const T xt49 = nt_cvt<T>(x[49]);
    const T xt50 = nt_cvt<T>(x[50]);
    const T xt51 = nt_cvt<T>(x[51]);
    const T xt52 = nt_cvt<T>(x[52]);
    const T xt53 = nt_cvt<T>(x[53]);
    const T xt54 = nt_cvt<T>(x[54]);
    const T xt55 = nt_cvt<T>(x[55]);
    const T xt56 = nt_cvt<T>(x[56]);
    const T cs1 = nt_scale<T>(nt_exp_hi(x[1]), fh);
    const T cs2 = nt_scale<T>(nt_exp_hi(x[2]), fh);
    const T cs4 = nt_scale<T>(nt_exp_hi(x[4]), fh);
    const T cs5 = nt_scale<T>(nt_exp_hi(x[5]), fh);
    const T cs7 = nt_scale<T>(nt_exp_hi(x[7]), fh);
    const T cs8 = nt_scale<T>(nt_exp_hi(x[8]), fh);
    const T cs12 = nt_scale<T>(nt_exp_hi(x[12]), fh);
    const T cs13 = nt_scale<T>(nt_exp_hi(x[13]), fh);
    const T cs14 = nt_scale<T>(nt_exp_hi(x[14]), fh);
    const T cs15 = nt_scale<T>(nt_exp_hi(x[15]), fh);
    const T cs16 = nt_scale<T>(nt_exp_hi(x[16]), fh);
    const T cs19 = nt_scale<T>(nt_exp_hi(x[19]), fh);
    const T cs27 = nt_scale<T>(nt_exp_hi(x[27]), fh);
    const T cs28 = nt_scale<T>(nt_exp_hi(x[28]), fh);
    const T cs29 = nt_scale<T>(nt_exp_hi(x[29]), fh);
    const T cs30 = nt_scale<T>(nt_exp_hi(x[30]), fh);
    const T cs31 = nt_scale<T>(nt_exp_hi(x[31]), fh);
    const T cs32 = nt_scale<T>(nt_exp_hi(x[32]), fh);
    const T cs33 = nt_scale<T>(nt_exp_hi(x[33]), fh);
    const T cs34 = nt_scale<T>(nt_exp_hi(x[34]), fh);
    const T cs35 = nt_scale<T>(nt_exp_hi(x[35]), fh);
    const T cs36 = nt_scale<T>(nt_exp_hi(x[36]), fh);
    const T cs37 = nt_scale<T>(nt_exp_hi(x[37]), fh);
    const T cs38 = nt_scale<T>(nt_exp_hi(x[38]), fh);
    const T cs42 = nt_scale<T>(nt_exp_hi(x[42]), fh);
    const T cs43 = nt_scale<T>(nt_exp_hi(x[43]), fh);
    const T cs44 = nt_scale<T>(nt_exp_hi(x[44]), fh);
    const T cs45 = nt_scale<T>(nt_exp_hi(x[45]), fh);
    const T cs46 = nt_scale<T>(nt_exp_hi(x[46]), fh);
    const T cs47 = nt_scale<T>(nt_exp_hi(x[47]), fh);
    const T cs48 = nt_scale<T>(nt_exp_hi(x[48]), fh);
    const T cs49 = nt_scale<T>(nt_exp_hi(x[49]), fh);
    const T cs50 = nt_scale<T>(nt_exp_hi(x[50]), fh);
    const T cs52 = nt_scale<T>(nt_exp_hi(x[52]), fh);
    const T cs53 = nt_scale<T>(nt_exp_hi(x[53]), fh);
    const T cs55 = nt_scale<T>(nt_exp_hi(x[55]), fh);
    const T cs56 = nt_scale<T>(nt_exp_hi(x[56]), fh);
    {  // row 1
    const T rs1 = nt_rscale<T>(nt_exp_hi(x[1]), fh);
        const T nj1_c0 = F.dt*xt1;
        J[157] = (F.dt*(K[K_c1a]*xt42 + K[K_c1b]*xt42 + K[K_c1c]*xt42 + K[K_c2]*xt43 + K[K_d5]*xt44) + T(1)) * (cs1 * rs1);
        J[156] = (nj1_c0*(K[K_c1a] + K[K_c1b] + K[K_c1c])) * (cs42 * rs1);
        J[159] = (K[K_c2]*nj1_c0) * (cs43 * rs1);
        J[158] = (K[K_d5]*nj1_c0) * (cs44 * rs1);
    }
    {  // row 2
    const T rs2 = nt_rscale<T>(nt_exp_hi(x[2]), fh);
        const T nj2_c0 = F.dt*xt43;
        const T nj2_c1 = F.dt*F.parth2o;
        const T nj2_c2 = F.parthno3*K[K_b27];
        const T nj2_c3 = F.parthcl*K[K_d11];
        J[261] = (-K[K_c2]*nj2_c0) * (cs1 * rs2);
        J[266] = (nj2_c1*(K[K_a1et]*xt42 + tj[J_h2o]) + T(1)) * (cs2 * rs2);
        J[260] = (-nj2_c0*nj2_c2) * (cs4 * rs2);
        J[265] = (-nj2_c0*nj2_c3) * (cs12 * rs2);
        J[262] = (-K[K_a30]*nj2_c0) * (cs16 * rs2);
        J[264] = (-K[K_c8]*nj2_c0) * (cs27 * rs2);
        J[258] = (-F.dt*(K[K_c17a]*xt43 + K[K_c17b]*xt43)) * (cs29 * rs2);
        J[259] = (K[K_a1et]*nj2_c1*xt2) * (cs42 * rs2);
        J[267] = (-F.dt*(F.h2*K[K_a19] + K[K_a17]*xt47 + K[K_a30]*xt16 + T(2)*K[K_a31]*xt43 + K[K_c17a]*xt29 + K[K_c17b]*xt29 + K[K_c2]*xt1 + K[K_c8]*xt27 + nj2_c2*xt4 + nj2_c3*xt12)) * (cs43 * rs2);
        J[268] = (-F.dt*(K[K_a17]*xt43 + T(1.6e-12)*xt55)) * (cs47 * rs2);
        J[263] = (-T(1.6e-12)*F.dt*xt47) * (cs55 * rs2);
    }
    {  // row 4
    const T rs4 = nt_rscale<T>(nt_exp_hi(x[4]), fh);
        const T nj4_c0 = T(2)*het[2];
        const T nj4_c1 = F.dt*K[K_b22];
        J[122] = (-F.dt*(het[0]*xt13 + het[5]*xt19 + nj4_c0*xt5)) * (cs2 * rs4);
        J[120] = (F.dt*(F.parthno3*(K[K_b27]*xt43 + tj[J_hno3]) + F.rain_hno3) + T(1)) * (cs4 * rs4);
        J[118] = (-F.dt*(het[3]*xt12 + nj4_c0*xt2)) * (cs5 * rs4);
        J[121] = (-F.dt*(het[1]*xt13 + het[3]*xt5)) * (cs12 * rs4);
        J[119] = (-F.dt*(het[0]*xt2 + het[1]*xt12)) * (cs13 * rs4);
        J[117] = (-F.dt*het[5]*xt2) * (cs19 * rs4);
        J[124] = (F.dt*F.parthno3*K[K_b27]*xt4 - nj4_c1*xt48) * (cs43 * rs4);
        J[123] = (-nj4_c1*xt43) * (cs48 * rs4);
    }
    {  // row 6
    const T rs6 = nt_rscale<T>(nt_exp_hi(x[6]), fh);
        const T nj6_c0 = T(3)*xt42;
        const T nj6_c1 = T(2)*K[K_d91];
        const T nj6_c2 = T(4)*K[K_d93];
        const T nj6_c3 = T(3)*K[K_d94];
        J[9] = (F.dt*F.rain_hcl) * (cs12 * rs6);
        J[7] = (-F.dt*(K[K_d90]*nj6_c0 + T(3)*tj[J_cfc11])) * (cs30 * rs6);
        J[4] = (-F.dt*(nj6_c1*xt42 + T(2)*tj[J_cfc12])) * (cs31 * rs6);
        J[0] = (-F.dt*(K[K_d92]*nj6_c0 + T(3)*tj[J_cfc113])) * (cs32 * rs6);
        J[2] = (-F.dt*(nj6_c2*xt42 + T(4)*tj[J_ccl4])) * (cs33 * rs6);
        J[6] = (-F.dt*(nj6_c3*xt43 + T(3)*tj[J_ch3ccl3])) * (cs34 * rs6);
        J[5] = (-F.dt*(K[K_d95]*xt43 + tj[J_ch3cl])) * (cs35 * rs6);
        J[3] = (-F.dt*(K[K_d96]*xt42 + K[K_d97]*xt43 + tj[J_hcfc22])) * (cs36 * rs6);
        J[1] = (-F.dt*(K[K_e52]*xt42 + tj[J_h1211])) * (cs38 * rs6);
        J[8] = (-F.dt*(T(3)*K[K_d90]*xt30 + T(3)*K[K_d92]*xt32 + K[K_d96]*xt36 + K[K_e52]*xt38 + nj6_c1*xt31 + nj6_c2*xt33)) * (cs42 * rs6);
        J[10] = (-F.dt*(K[K_d95]*xt35 + K[K_d97]*xt36 + nj6_c3*xt34)) * (cs43 * rs6);
    }
    {  // row 15
    const T rs15 = nt_rscale<T>(nt_exp_hi(x[15]), fh);
        J[63] = (-F.dt*(het[1]*xt13 + het[4]*xt14)) * (cs12 * rs15);
        J[61] = (-F.dt*het[1]*xt12) * (cs13 * rs15);
        J[62] = (-F.dt*(K[K_d37]*xt44 + het[4]*xt12)) * (cs14 * rs15);
        J[60] = (F.dt*tj[J_cl2] + T(1)) * (cs15 * rs15);
        J[64] = (-F.dt*K[K_d37]*xt14) * (cs44 * rs15);
        J[65] = (-T(2)*F.dt*K[K_d62]*xt52) * (cs52 * rs15);
    }
    {  // row 28
    const T rs28 = nt_rscale<T>(nt_exp_hi(x[28]), fh);
        const T nj28_c0 = T(2)*K[K_c14]*xt28;
        const T nj28_c1 = F.dt*K[K_c17a];
        const T nj28_c2 = F.dt*xt28;
        J[212] = (F.dt*nj28_c0 + F.dt*(K[K_c18]*xt52 + K[K_c5]*xt49 + K[K_c7]*xt47 + nj28_c0) + T(1)) * (cs28 * rs28);
        J[210] = (-nj28_c1*xt43) * (cs29 * rs28);
        J[213] = (-nj28_c1*xt29) * (cs43 * rs28);
        J[214] = (K[K_c7]*nj28_c2) * (cs47 * rs28);
        J[215] = (K[K_c5]*nj28_c2) * (cs49 * rs28);
        J[216] = (K[K_c18]*nj28_c2) * (cs52 * rs28);
        J[211] = (-F.dt*F.o2*K[K_c4]) * (cs56 * rs28);
    }
    {  // row 29
    const T rs29 = nt_rscale<T>(nt_exp_hi(x[29]), fh);
        const T nj29_c0 = F.dt*K[K_c7];
        J[35] = (-nj29_c0*xt47) * (cs28 * rs29);
        J[34] = (F.dt*(K[K_c17a]*xt43 + K[K_c17b]*xt43 + tj[J_ch3o2h]) + T(1)) * (cs29 * rs29);
        J[36] = (F.dt*xt29*(K[K_c17a] + K[K_c17b])) * (cs43 * rs29);
        J[37] = (-nj29_c0*xt28) * (cs47 * rs29);
    }
    {  // row 30
    const T rs30 = nt_rscale<T>(nt_exp_hi(x[30]), fh);
        J[95] = (F.dt*(K[K_d90]*xt42 + tj[J_cfc11]) + T(1)) * (cs30 * rs30);
        J[96] = (F.dt*K[K_d90]*xt30) * (cs42 * rs30);
    }
    {  // row 32
    const T rs32 = nt_rscale<T>(nt_exp_hi(x[32]), fh);
        J[18] = (F.dt*(K[K_d92]*xt42 + tj[J_cfc113]) + T(1)) * (cs32 * rs32);
        J[19] = (F.dt*K[K_d92]*xt32) * (cs42 * rs32);
    }
    {  // row 37
    const T rs37 = nt_rscale<T>(nt_exp_hi(x[37]), fh);
        const T nj37_c0 = F.dt*xt37;
        J[52] = (F.dt*(K[K_e50]*xt42 + K[K_e51]*xt43 + tj[J_ch3br]) + T(1)) * (cs37 * rs37);
        J[53] = (K[K_e50]*nj37_c0) * (cs42 * rs37);
        J[54] = (K[K_e51]*nj37_c0) * (cs43 * rs37);
    }
    {  // row 38
    const T rs38 = nt_rscale<T>(nt_exp_hi(x[38]), fh);
        J[30] = (F.dt*(K[K_e52]*xt42 + tj[J_h1211]) + T(1)) * (cs38 * rs38);
        J[31] = (F.dt*K[K_e52]*xt38) * (cs42 * rs38);
    }
    {  // row 46
    const T rs46 = nt_rscale<T>(nt_exp_hi(x[46]), fh);
        J[355] = (T(-1)) * (cs7 * rs46);
        J[358] = T(0);
        J[357] = T(0);
        J[359] = T(0);
        J[360] = T(0);
        J[356] = T(0);
    }
    {  // row 47
    const T rs47 = nt_rscale<T>(nt_exp_hi(x[47]), fh);
        J[342] = T(0);
        J[343] = T(0);
        J[345] = T(0);
        J[350] = T(0);
        J[347] = T(0);
        J[346] = T(0);
        J[352] = T(0);
        J[351] = (T(1)) * (cs47 * rs47);
        J[353] = T(0);
        J[349] = T(0);
        J[354] = T(0);
        J[348] = T(0);
        J[344] = T(0);
    }
    {  // row 55
    const T rs55 = nt_rscale<T>(nt_exp_hi(x[55]), fh);
        J[205] = T(0);
        J[207] = T(0);
        J[206] = T(0);
        J[209] = T(0);
        J[208] = T(0);
    }
}

// residual rows of group g of 4 (night equations)
template <typename T, typename FF, typename PK, typename PC, typename PX, typename PR>
__device__ __forceinline__ void nt_residual_night_w4(int g, const FF& F, PK K, PK tj, PK het, PC ck0, PX x, PR R) {
    switch (g) {
        case 0: nt_residual_night_w4_0<T>(F, K, tj, het, ck0, x, R); break;
        case 1: nt_residual_night_w4_1<T>(F, K, tj, het, ck0, x, R); break;
        case 2: nt_residual_night_w4_2<T>(F, K, tj, het, ck0, x, R); break;
        case 3: nt_residual_night_w4_3<T>(F, K, tj, het, ck0, x, R); break;
        default: break;
    }
}
// Jacobian rows of group g of 4 (night equations)
template <typename T, typename FF, typename PK, typename PJ>
__device__ __forceinline__ void nt_jacobian_night_w4(int g, const FF& F, PK K, PK tj, PK het, const double* __restrict__ x, double floor_, PJ J) {
    switch (g) {
        case 0: nt_jacobian_night_w4_0<T>(F, K, tj, het, x, floor_, J); break;
        case 1: nt_jacobian_night_w4_1<T>(F, K, tj, het, x, floor_, J); break;
        case 2: nt_jacobian_night_w4_2<T>(F, K, tj, het, x, floor_, J); break;
        case 3: nt_jacobian_night_w4_3<T>(F, K, tj, het, x, floor_, J); break;
        default: break;
    }
}

// Crout factorisation, row by row in elimination order, of the stored scaled
// matrix, with the forward substitution fused: row t is read into registers
// w, reduced by the earlier unit-upper rows U~(k,:), its pivot p = w_t taken
// (a zero or non-finite pivot replaced by +-tiny: the FP64 residual corrects
// the step), z_t = (z_t - sum_k w_k z_k) / p and U~(t,j) = w_j / p stored;
// then the back substitution. z (original numbering, registers or a view):
// right-hand side in, solution out. L is never stored. NT_FENCE keeps each
// row's shared-memory loads in that row (hoisted loads would hold registers).
template <typename T, typename PJ, typename PZ>
__device__ __forceinline__ void nt_factor_solve(PJ J, PZ z, T tiny) {
    NT_FENCE();
    {  // row 0: unknown 6
        T w0 = T(1.0);
        T w2 = J[0];
        T w5 = J[1];
        T w6 = J[2];
        T w9 = J[3];
        T w10 = J[4];
        T w16 = J[5];
        T w23 = J[6];
        T w24 = J[7];
        T w26 = J[8];
        T w44 = J[9];
        T w52 = J[10];
        T zt = z[6];
        T p = w0; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[6] = zt * d;
        J[0] = w2 * d;
        J[1] = w5 * d;
        J[2] = w6 * d;
        J[3] = w9 * d;
        J[4] = w10 * d;
        J[5] = w16 * d;
        J[6] = w23 * d;
        J[7] = w24 * d;
        J[8] = w26 * d;
        J[9] = w44 * d;
        J[10] = w52 * d;
    }
    NT_FENCE();
    {  // row 1: unknown 40
        T w1 = T(1.0);
        T w5 = J[11];
        T w12 = J[12];
        T w13 = J[13];
        T w26 = J[14];
        T w30 = J[15];
        T w37 = J[16];
        T w52 = J[17];
        T zt = z[40];
        T p = w1; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[40] = zt * d;
        J[11] = w5 * d;
        J[12] = w12 * d;
        J[13] = w13 * d;
        J[14] = w26 * d;
        J[15] = w30 * d;
        J[16] = w37 * d;
        J[17] = w52 * d;
    }
    NT_FENCE();
    {  // row 2: unknown 32
        T w2 = J[18];
        T w26 = J[19];
        T zt = z[32];
        T p = w2; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[32] = zt * d;
        J[18] = w26 * d;
    }
    NT_FENCE();
    {  // row 3: unknown 3
        T w3 = T(1.0);
        T w19 = J[20];
        T w20 = J[21];
        T w26 = J[22];
        T w29 = J[23];
        T w55 = J[24];
        T zt = z[3];
        T p = w3; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[3] = zt * d;
        J[19] = w19 * d;
        J[20] = w20 * d;
        J[21] = w26 * d;
        J[22] = w29 * d;
        J[23] = w55 * d;
    }
    NT_FENCE();
    {  // row 4: unknown 17
        T w4 = J[25];
        T w18 = J[26];
        T w44 = J[27];
        T w46 = J[28];
        T w49 = J[29];
        T zt = z[17];
        T p = w4; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[17] = zt * d;
        J[24] = w18 * d;
        J[25] = w44 * d;
        J[26] = w46 * d;
        J[27] = w49 * d;
    }
    NT_FENCE();
    {  // row 5: unknown 38
        T w5 = J[30];
        T w26 = J[31];
        T zt = z[38];
        T p = w5; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[38] = zt * d;
        J[28] = w26 * d;
    }
    NT_FENCE();
    {  // row 6: unknown 33
        T w6 = J[32];
        T w26 = J[33];
        T zt = z[33];
        T p = w6; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[33] = zt * d;
        J[29] = w26 * d;
    }
    NT_FENCE();
    {  // row 7: unknown 11
        T w7 = T(1.0);
        T zt = z[11];
        T p = w7; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[11] = zt * d;
    }
    NT_FENCE();
    {  // row 8: unknown 29
        T w8 = J[34];
        T w41 = J[35];
        T w52 = J[36];
        T w53 = J[37];
        T zt = z[29];
        T p = w8; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[29] = zt * d;
        J[30] = w41 * d;
        J[31] = w52 * d;
        J[32] = w53 * d;
    }
    NT_FENCE();
    {  // row 9: unknown 36
        T w9 = J[38];
        T w26 = J[39];
        T w52 = J[40];
        T zt = z[36];
        T p = w9; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[36] = zt * d;
        J[33] = w26 * d;
        J[34] = w52 * d;
    }
    NT_FENCE();
    {  // row 10: unknown 31
        T w10 = J[41];
        T w26 = J[42];
        T zt = z[31];
        T p = w10; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[31] = zt * d;
        J[35] = w26 * d;
    }
    NT_FENCE();
    {  // row 11: unknown 26
        T w11 = J[43];
        T w21 = J[44];
        T w35 = J[45];
        T w37 = J[46];
        T w44 = J[47];
        T w50 = J[48];
        T w56 = J[49];
        T zt = z[26];
        T p = w11; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[26] = zt * d;
        J[36] = w21 * d;
        J[37] = w35 * d;
        J[38] = w37 * d;
        J[39] = w44 * d;
        J[40] = w50 * d;
        J[41] = w56 * d;
    }
    NT_FENCE();
    {  // row 12: unknown 39
        T w12 = J[50];
        T w26 = J[51];
        T zt = z[39];
        T p = w12; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[39] = zt * d;
        J[42] = w26 * d;
    }
    NT_FENCE();
    {  // row 13: unknown 37
        T w13 = J[52];
        T w26 = J[53];
        T w52 = J[54];
        T zt = z[37];
        T p = w13; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[37] = zt * d;
        J[43] = w26 * d;
        J[44] = w52 * d;
    }
    NT_FENCE();
    {  // row 14: unknown 19
        T w14 = J[55];
        T w45 = J[56];
        T w46 = J[57];
        T w47 = J[58];
        T w50 = J[59];
        T zt = z[19];
        T p = w14; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[19] = zt * d;
        J[45] = w45 * d;
        J[46] = w46 * d;
        J[47] = w47 * d;
        J[48] = w50 * d;
    }
    NT_FENCE();
    {  // row 15: unknown 15
        T w15 = J[60];
        T w22 = J[61];
        T w35 = J[62];
        T w44 = J[63];
        T w49 = J[64];
        T w56 = J[65];
        T zt = z[15];
        T p = w15; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[15] = zt * d;
        J[49] = w22 * d;
        J[50] = w35 * d;
        J[51] = w44 * d;
        J[52] = w49 * d;
        J[53] = w56 * d;
    }
    NT_FENCE();
    {  // row 16: unknown 35
        T w16 = J[66];
        T w52 = J[67];
        T zt = z[35];
        T p = w16; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[35] = zt * d;
        J[54] = w52 * d;
    }
    NT_FENCE();
    {  // row 17: unknown 54
        T w17 = T(1.0);
        T w43 = J[68];
        T w46 = J[69];
        T w54 = J[70];
        T zt = z[54];
        T p = w17; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[54] = zt * d;
        J[55] = w43 * d;
        J[56] = w46 * d;
        J[57] = w54 * d;
    }
    NT_FENCE();
    {  // row 18: unknown 5
        T w17 = J[71];
        T w18 = J[72];
        T w43 = T(0);
        T w44 = J[73];
        T w45 = J[74];
        T w46 = J[75];
        T w54 = T(0);
        T zt = z[5];
        zt -= w17 * z[54];
        w43 -= w17 * J[55];
        w46 -= w17 * J[56];
        w54 -= w17 * J[57];
        T p = w18; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[5] = zt * d;
        J[58] = w43 * d;
        J[59] = w44 * d;
        J[60] = w45 * d;
        J[61] = w46 * d;
        J[62] = w54 * d;
    }
    NT_FENCE();
    {  // row 19: unknown 0
        T w19 = J[76];
        T w26 = J[77];
        T zt = z[0];
        T p = w19; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[0] = zt * d;
        J[63] = w26 * d;
    }
    NT_FENCE();
    {  // row 20: unknown 51
        T w20 = T(1.0);
        T w55 = J[78];
        T zt = z[51];
        T p = w20; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[51] = zt * d;
        J[64] = w55 * d;
    }
    NT_FENCE();
    {  // row 21: unknown 25
        T w14 = J[79];
        T w21 = J[80];
        T w37 = J[81];
        T w44 = J[82];
        T w45 = J[83];
        T w46 = T(0);
        T w47 = J[84];
        T w50 = J[85];
        T w53 = J[86];
        T zt = z[25];
        zt -= w14 * z[19];
        w45 -= w14 * J[45];
        w46 -= w14 * J[46];
        w47 -= w14 * J[47];
        w50 -= w14 * J[48];
        T p = w21; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[25] = zt * d;
        J[65] = w37 * d;
        J[66] = w44 * d;
        J[67] = w45 * d;
        J[68] = w46 * d;
        J[69] = w47 * d;
        J[70] = w50 * d;
        J[71] = w53 * d;
    }
    NT_FENCE();
    {  // row 22: unknown 13
        T w22 = J[87];
        T w44 = J[88];
        T w45 = J[89];
        T w46 = J[90];
        T w47 = J[91];
        T w56 = J[92];
        T zt = z[13];
        T p = w22; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[13] = zt * d;
        J[72] = w44 * d;
        J[73] = w45 * d;
        J[74] = w46 * d;
        J[75] = w47 * d;
        J[76] = w56 * d;
    }
    NT_FENCE();
    {  // row 23: unknown 34
        T w23 = J[93];
        T w52 = J[94];
        T zt = z[34];
        T p = w23; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[34] = zt * d;
        J[77] = w52 * d;
    }
    NT_FENCE();
    {  // row 24: unknown 30
        T w24 = J[95];
        T w26 = J[96];
        T zt = z[30];
        T p = w24; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[30] = zt * d;
        J[78] = w26 * d;
    }
    NT_FENCE();
    {  // row 25: unknown 24
        T w25 = J[97];
        T w56 = J[98];
        T zt = z[24];
        T p = w25; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[24] = zt * d;
        J[79] = w56 * d;
    }
    NT_FENCE();
    {  // row 26: unknown 42
        T w26 = T(1.0);
        T w54 = J[99];
        T zt = z[42];
        T p = w26; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[42] = zt * d;
        J[80] = w54 * d;
    }
    NT_FENCE();
    {  // row 27: unknown 9
        T w27 = J[100];
        T w50 = J[101];
        T w56 = J[102];
        T zt = z[9];
        T p = w27; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[9] = zt * d;
        J[81] = w50 * d;
        J[82] = w56 * d;
    }
    NT_FENCE();
    {  // row 28: unknown 7
        T w11 = J[103];
        T w21 = J[104];
        T w22 = J[105];
        T w28 = T(1.0);
        T w35 = J[106];
        T w37 = T(0);
        T w40 = J[107];
        T w41 = J[108];
        T w44 = T(0);
        T w45 = T(0);
        T w46 = J[109];
        T w47 = J[110];
        T w50 = J[111];
        T w52 = J[112];
        T w53 = J[113];
        T w54 = J[114];
        T w55 = J[115];
        T w56 = J[116];
        T zt = z[7];
        zt -= w11 * z[26];
        w21 -= w11 * J[36];
        w35 -= w11 * J[37];
        w37 -= w11 * J[38];
        w44 -= w11 * J[39];
        w50 -= w11 * J[40];
        w56 -= w11 * J[41];
        zt -= w21 * z[25];
        w37 -= w21 * J[65];
        w44 -= w21 * J[66];
        w45 -= w21 * J[67];
        w46 -= w21 * J[68];
        w47 -= w21 * J[69];
        w50 -= w21 * J[70];
        w53 -= w21 * J[71];
        zt -= w22 * z[13];
        w44 -= w22 * J[72];
        w45 -= w22 * J[73];
        w46 -= w22 * J[74];
        w47 -= w22 * J[75];
        w56 -= w22 * J[76];
        T p = w28; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[7] = zt * d;
        J[83] = w35 * d;
        J[84] = w37 * d;
        J[85] = w40 * d;
        J[86] = w41 * d;
        J[87] = w44 * d;
        J[88] = w45 * d;
        J[89] = w46 * d;
        J[90] = w47 * d;
        J[91] = w50 * d;
        J[92] = w52 * d;
        J[93] = w53 * d;
        J[94] = w54 * d;
        J[95] = w55 * d;
        J[96] = w56 * d;
    }
    NT_FENCE();
    {  // row 29: unknown 4
        T w14 = J[117];
        T w18 = J[118];
        T w22 = J[119];
        T w29 = J[120];
        T w43 = T(0);
        T w44 = J[121];
        T w45 = J[122];
        T w46 = J[123];
        T w47 = T(0);
        T w50 = T(0);
        T w52 = J[124];
        T w54 = T(0);
        T w56 = T(0);
        T zt = z[4];
        zt -= w14 * z[19];
        w45 -= w14 * J[45];
        w46 -= w14 * J[46];
        w47 -= w14 * J[47];
        w50 -= w14 * J[48];
        zt -= w18 * z[5];
        w43 -= w18 * J[58];
        w44 -= w18 * J[59];
        w45 -= w18 * J[60];
        w46 -= w18 * J[61];
        w54 -= w18 * J[62];
        zt -= w22 * z[13];
        w44 -= w22 * J[72];
        w45 -= w22 * J[73];
        w46 -= w22 * J[74];
        w47 -= w22 * J[75];
        w56 -= w22 * J[76];
        T p = w29; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[4] = zt * d;
        J[97] = w43 * d;
        J[98] = w44 * d;
        J[99] = w45 * d;
        J[100] = w46 * d;
        J[101] = w47 * d;
        J[102] = w50 * d;
        J[103] = w52 * d;
        J[104] = w54 * d;
        J[105] = w56 * d;
    }
    NT_FENCE();
    {  // row 30: unknown 41
        T w30 = J[125];
        T w52 = J[126];
        T zt = z[41];
        T p = w30; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[41] = zt * d;
        J[106] = w52 * d;
    }
    NT_FENCE();
    {  // row 31: unknown 22
        T w2 = J[127];
        T w4 = J[128];
        T w6 = J[129];
        T w9 = J[130];
        T w10 = J[131];
        T w11 = J[132];
        T w15 = J[133];
        T w16 = J[134];
        T w18 = T(0);
        T w21 = T(0);
        T w22 = J[135];
        T w23 = J[136];
        T w24 = J[137];
        T w25 = J[138];
        T w26 = J[139];
        T w27 = J[140];
        T w31 = T(1.0);
        T w33 = J[141];
        T w35 = J[142];
        T w37 = T(0);
        T w42 = J[143];
        T w43 = T(0);
        T w44 = J[144];
        T w45 = T(0);
        T w46 = J[145];
        T w47 = J[146];
        T w49 = J[147];
        T w50 = J[148];
        T w52 = J[149];
        T w53 = J[150];
        T w54 = T(0);
        T w56 = J[151];
        T zt = z[22];
        zt -= w2 * z[32];
        w26 -= w2 * J[18];
        zt -= w4 * z[17];
        w18 -= w4 * J[24];
        w44 -= w4 * J[25];
        w46 -= w4 * J[26];
        w49 -= w4 * J[27];
        zt -= w6 * z[33];
        w26 -= w6 * J[29];
        zt -= w9 * z[36];
        w26 -= w9 * J[33];
        w52 -= w9 * J[34];
        zt -= w10 * z[31];
        w26 -= w10 * J[35];
        zt -= w11 * z[26];
        w21 -= w11 * J[36];
        w35 -= w11 * J[37];
        w37 -= w11 * J[38];
        w44 -= w11 * J[39];
        w50 -= w11 * J[40];
        w56 -= w11 * J[41];
        zt -= w15 * z[15];
        w22 -= w15 * J[49];
        w35 -= w15 * J[50];
        w44 -= w15 * J[51];
        w49 -= w15 * J[52];
        w56 -= w15 * J[53];
        zt -= w16 * z[35];
        w52 -= w16 * J[54];
        zt -= w18 * z[5];
        w43 -= w18 * J[58];
        w44 -= w18 * J[59];
        w45 -= w18 * J[60];
        w46 -= w18 * J[61];
        w54 -= w18 * J[62];
        zt -= w21 * z[25];
        w37 -= w21 * J[65];
        w44 -= w21 * J[66];
        w45 -= w21 * J[67];
        w46 -= w21 * J[68];
        w47 -= w21 * J[69];
        w50 -= w21 * J[70];
        w53 -= w21 * J[71];
        zt -= w22 * z[13];
        w44 -= w22 * J[72];
        w45 -= w22 * J[73];
        w46 -= w22 * J[74];
        w47 -= w22 * J[75];
        w56 -= w22 * J[76];
        zt -= w23 * z[34];
        w52 -= w23 * J[77];
        zt -= w24 * z[30];
        w26 -= w24 * J[78];
        zt -= w25 * z[24];
        w56 -= w25 * J[79];
        zt -= w26 * z[42];
        w54 -= w26 * J[80];
        zt -= w27 * z[9];
        w50 -= w27 * J[81];
        w56 -= w27 * J[82];
        T p = w31; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[22] = zt * d;
        J[107] = w33 * d;
        J[108] = w35 * d;
        J[109] = w37 * d;
        J[110] = w42 * d;
        J[111] = w43 * d;
        J[112] = w44 * d;
        J[113] = w45 * d;
        J[114] = w46 * d;
        J[115] = w47 * d;
        J[116] = w49 * d;
        J[117] = w50 * d;
        J[118] = w52 * d;
        J[119] = w53 * d;
        J[120] = w54 * d;
        J[121] = w56 * d;
    }
    NT_FENCE();
    {  // row 32: unknown 21
        T w32 = J[152];
        T w46 = J[153];
        T w52 = J[154];
        T w53 = J[155];
        T zt = z[21];
        T p = w32; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[21] = zt * d;
        J[122] = w46 * d;
        J[123] = w52 * d;
        J[124] = w53 * d;
    }
    NT_FENCE();
    {  // row 33: unknown 1
        T w26 = J[156];
        T w33 = J[157];
        T w49 = J[158];
        T w52 = J[159];
        T w54 = T(0);
        T zt = z[1];
        zt -= w26 * z[42];
        w54 -= w26 * J[80];
        T p = w33; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[1] = zt * d;
        J[125] = w49 * d;
        J[126] = w52 * d;
        J[127] = w54 * d;
    }
    NT_FENCE();
    {  // row 34: unknown 8
        T w34 = J[160];
        T w42 = J[161];
        T w47 = J[162];
        T w49 = J[163];
        T w51 = J[164];
        T w52 = J[165];
        T zt = z[8];
        T p = w34; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[8] = zt * d;
        J[128] = w42 * d;
        J[129] = w47 * d;
        J[130] = w49 * d;
        J[131] = w51 * d;
        J[132] = w52 * d;
    }
    NT_FENCE();
    {  // row 35: unknown 14
        T w22 = J[166];
        T w35 = J[167];
        T w37 = J[168];
        T w44 = J[169];
        T w45 = J[170];
        T w46 = T(0);
        T w47 = J[171];
        T w49 = J[172];
        T w52 = J[173];
        T w53 = J[174];
        T w56 = J[175];
        T zt = z[14];
        zt -= w22 * z[13];
        w44 -= w22 * J[72];
        w45 -= w22 * J[73];
        w46 -= w22 * J[74];
        w47 -= w22 * J[75];
        w56 -= w22 * J[76];
        T p = w35; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[14] = zt * d;
        J[133] = w37 * d;
        J[134] = w44 * d;
        J[135] = w45 * d;
        J[136] = w46 * d;
        J[137] = w47 * d;
        J[138] = w49 * d;
        J[139] = w52 * d;
        J[140] = w53 * d;
        J[141] = w56 * d;
    }
    NT_FENCE();
    {  // row 36: unknown 56
        T w26 = J[176];
        T w33 = J[177];
        T w36 = T(1.0);
        T w47 = J[178];
        T w49 = J[179];
        T w52 = J[180];
        T w54 = T(0);
        T zt = z[56];
        zt -= w26 * z[42];
        w54 -= w26 * J[80];
        zt -= w33 * z[1];
        w49 -= w33 * J[125];
        w52 -= w33 * J[126];
        w54 -= w33 * J[127];
        T p = w36; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[56] = zt * d;
        J[142] = w47 * d;
        J[143] = w49 * d;
        J[144] = w52 * d;
        J[145] = w54 * d;
    }
    NT_FENCE();
    {  // row 37: unknown 18
        T w21 = J[181];
        T w26 = J[182];
        T w35 = J[183];
        T w37 = J[184];
        T w42 = J[185];
        T w44 = T(0);
        T w45 = T(0);
        T w46 = T(0);
        T w47 = T(0);
        T w49 = T(0);
        T w50 = T(0);
        T w51 = J[186];
        T w52 = J[187];
        T w53 = J[188];
        T w54 = T(0);
        T w56 = T(0);
        T zt = z[18];
        zt -= w21 * z[25];
        w37 -= w21 * J[65];
        w44 -= w21 * J[66];
        w45 -= w21 * J[67];
        w46 -= w21 * J[68];
        w47 -= w21 * J[69];
        w50 -= w21 * J[70];
        w53 -= w21 * J[71];
        zt -= w26 * z[42];
        w54 -= w26 * J[80];
        zt -= w35 * z[14];
        w37 -= w35 * J[133];
        w44 -= w35 * J[134];
        w45 -= w35 * J[135];
        w46 -= w35 * J[136];
        w47 -= w35 * J[137];
        w49 -= w35 * J[138];
        w52 -= w35 * J[139];
        w53 -= w35 * J[140];
        w56 -= w35 * J[141];
        T p = w37; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[18] = zt * d;
        J[146] = w42 * d;
        J[147] = w44 * d;
        J[148] = w45 * d;
        J[149] = w46 * d;
        J[150] = w47 * d;
        J[151] = w49 * d;
        J[152] = w50 * d;
        J[153] = w51 * d;
        J[154] = w52 * d;
        J[155] = w53 * d;
        J[156] = w54 * d;
        J[157] = w56 * d;
    }
    NT_FENCE();
    {  // row 38: unknown 16
        T w38 = J[189];
        T w52 = J[190];
        T w53 = J[191];
        T zt = z[16];
        T p = w38; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[16] = zt * d;
        J[158] = w52 * d;
        J[159] = w53 * d;
    }
    NT_FENCE();
    {  // row 39: unknown 23
        T w11 = J[192];
        T w14 = J[193];
        T w21 = J[194];
        T w26 = J[195];
        T w35 = T(0);
        T w37 = J[196];
        T w39 = T(1.0);
        T w42 = J[197];
        T w44 = T(0);
        T w45 = T(0);
        T w46 = J[198];
        T w47 = J[199];
        T w49 = T(0);
        T w50 = J[200];
        T w51 = J[201];
        T w52 = J[202];
        T w53 = J[203];
        T w54 = T(0);
        T w56 = J[204];
        T zt = z[23];
        zt -= w11 * z[26];
        w21 -= w11 * J[36];
        w35 -= w11 * J[37];
        w37 -= w11 * J[38];
        w44 -= w11 * J[39];
        w50 -= w11 * J[40];
        w56 -= w11 * J[41];
        zt -= w14 * z[19];
        w45 -= w14 * J[45];
        w46 -= w14 * J[46];
        w47 -= w14 * J[47];
        w50 -= w14 * J[48];
        zt -= w21 * z[25];
        w37 -= w21 * J[65];
        w44 -= w21 * J[66];
        w45 -= w21 * J[67];
        w46 -= w21 * J[68];
        w47 -= w21 * J[69];
        w50 -= w21 * J[70];
        w53 -= w21 * J[71];
        zt -= w26 * z[42];
        w54 -= w26 * J[80];
        zt -= w35 * z[14];
        w37 -= w35 * J[133];
        w44 -= w35 * J[134];
        w45 -= w35 * J[135];
        w46 -= w35 * J[136];
        w47 -= w35 * J[137];
        w49 -= w35 * J[138];
        w52 -= w35 * J[139];
        w53 -= w35 * J[140];
        w56 -= w35 * J[141];
        zt -= w37 * z[18];
        w42 -= w37 * J[146];
        w44 -= w37 * J[147];
        w45 -= w37 * J[148];
        w46 -= w37 * J[149];
        w47 -= w37 * J[150];
        w49 -= w37 * J[151];
        w50 -= w37 * J[152];
        w51 -= w37 * J[153];
        w52 -= w37 * J[154];
        w53 -= w37 * J[155];
        w54 -= w37 * J[156];
        w56 -= w37 * J[157];
        T p = w39; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[23] = zt * d;
        J[160] = w42 * d;
        J[161] = w44 * d;
        J[162] = w45 * d;
        J[163] = w46 * d;
        J[164] = w47 * d;
        J[165] = w49 * d;
        J[166] = w50 * d;
        J[167] = w51 * d;
        J[168] = w52 * d;
        J[169] = w53 * d;
        J[170] = w54 * d;
        J[171] = w56 * d;
    }
    NT_FENCE();
    {  // row 40: unknown 55
        T w34 = J[205];
        T w40 = T(1.0);
        T w42 = T(0);
        T w47 = J[206];
        T w49 = T(0);
        T w51 = T(0);
        T w52 = J[207];
        T w53 = J[208];
        T w54 = J[209];
        T zt = z[55];
        zt -= w34 * z[8];
        w42 -= w34 * J[128];
        w47 -= w34 * J[129];
        w49 -= w34 * J[130];
        w51 -= w34 * J[131];
        w52 -= w34 * J[132];
        T p = w40; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[55] = zt * d;
        J[172] = w42 * d;
        J[173] = w47 * d;
        J[174] = w49 * d;
        J[175] = w51 * d;
        J[176] = w52 * d;
        J[177] = w53 * d;
        J[178] = w54 * d;
    }
    NT_FENCE();
    {  // row 41: unknown 28
        T w8 = J[210];
        T w36 = J[211];
        T w41 = J[212];
        T w47 = T(0);
        T w49 = T(0);
        T w52 = J[213];
        T w53 = J[214];
        T w54 = T(0);
        T w55 = J[215];
        T w56 = J[216];
        T zt = z[28];
        zt -= w8 * z[29];
        w41 -= w8 * J[30];
        w52 -= w8 * J[31];
        w53 -= w8 * J[32];
        zt -= w36 * z[56];
        w47 -= w36 * J[142];
        w49 -= w36 * J[143];
        w52 -= w36 * J[144];
        w54 -= w36 * J[145];
        T p = w41; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[28] = zt * d;
        J[179] = w47 * d;
        J[180] = w49 * d;
        J[181] = w52 * d;
        J[182] = w53 * d;
        J[183] = w54 * d;
        J[184] = w55 * d;
        J[185] = w56 * d;
    }
    NT_FENCE();
    {  // row 42: unknown 27
        T w8 = J[217];
        T w26 = J[218];
        T w33 = J[219];
        T w36 = J[220];
        T w41 = J[221];
        T w42 = J[222];
        T w47 = J[223];
        T w49 = J[224];
        T w51 = J[225];
        T w52 = J[226];
        T w53 = T(0);
        T w54 = T(0);
        T w55 = J[227];
        T w56 = J[228];
        T zt = z[27];
        zt -= w8 * z[29];
        w41 -= w8 * J[30];
        w52 -= w8 * J[31];
        w53 -= w8 * J[32];
        zt -= w26 * z[42];
        w54 -= w26 * J[80];
        zt -= w33 * z[1];
        w49 -= w33 * J[125];
        w52 -= w33 * J[126];
        w54 -= w33 * J[127];
        zt -= w36 * z[56];
        w47 -= w36 * J[142];
        w49 -= w36 * J[143];
        w52 -= w36 * J[144];
        w54 -= w36 * J[145];
        zt -= w41 * z[28];
        w47 -= w41 * J[179];
        w49 -= w41 * J[180];
        w52 -= w41 * J[181];
        w53 -= w41 * J[182];
        w54 -= w41 * J[183];
        w55 -= w41 * J[184];
        w56 -= w41 * J[185];
        T p = w42; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[27] = zt * d;
        J[186] = w47 * d;
        J[187] = w49 * d;
        J[188] = w51 * d;
        J[189] = w52 * d;
        J[190] = w53 * d;
        J[191] = w54 * d;
        J[192] = w55 * d;
        J[193] = w56 * d;
    }
    NT_FENCE();
    {  // row 43: unknown 20
        T w4 = J[229];
        T w14 = J[230];
        T w17 = J[231];
        T w18 = J[232];
        T w19 = J[233];
        T w20 = J[234];
        T w22 = J[235];
        T w26 = J[236];
        T w29 = J[237];
        T w32 = J[238];
        T w43 = T(1.0);
        T w44 = T(0);
        T w45 = T(0);
        T w46 = J[239];
        T w47 = J[240];
        T w49 = J[241];
        T w50 = J[242];
        T w52 = J[243];
        T w53 = J[244];
        T w54 = T(0);
        T w55 = J[245];
        T w56 = J[246];
        T zt = z[20];
        zt -= w4 * z[17];
        w18 -= w4 * J[24];
        w44 -= w4 * J[25];
        w46 -= w4 * J[26];
        w49 -= w4 * J[27];
        zt -= w14 * z[19];
        w45 -= w14 * J[45];
        w46 -= w14 * J[46];
        w47 -= w14 * J[47];
        w50 -= w14 * J[48];
        zt -= w17 * z[54];
        w43 -= w17 * J[55];
        w46 -= w17 * J[56];
        w54 -= w17 * J[57];
        zt -= w18 * z[5];
        w43 -= w18 * J[58];
        w44 -= w18 * J[59];
        w45 -= w18 * J[60];
        w46 -= w18 * J[61];
        w54 -= w18 * J[62];
        zt -= w19 * z[0];
        w26 -= w19 * J[63];
        zt -= w20 * z[51];
        w55 -= w20 * J[64];
        zt -= w22 * z[13];
        w44 -= w22 * J[72];
        w45 -= w22 * J[73];
        w46 -= w22 * J[74];
        w47 -= w22 * J[75];
        w56 -= w22 * J[76];
        zt -= w26 * z[42];
        w54 -= w26 * J[80];
        zt -= w29 * z[4];
        w43 -= w29 * J[97];
        w44 -= w29 * J[98];
        w45 -= w29 * J[99];
        w46 -= w29 * J[100];
        w47 -= w29 * J[101];
        w50 -= w29 * J[102];
        w52 -= w29 * J[103];
        w54 -= w29 * J[104];
        w56 -= w29 * J[105];
        zt -= w32 * z[21];
        w46 -= w32 * J[122];
        w52 -= w32 * J[123];
        w53 -= w32 * J[124];
        T p = w43; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[20] = zt * d;
        J[194] = w44 * d;
        J[195] = w45 * d;
        J[196] = w46 * d;
        J[197] = w47 * d;
        J[198] = w49 * d;
        J[199] = w50 * d;
        J[200] = w52 * d;
        J[201] = w53 * d;
        J[202] = w54 * d;
        J[203] = w55 * d;
        J[204] = w56 * d;
    }
    NT_FENCE();
    {  // row 44: unknown 12
        T w18 = J[247];
        T w21 = J[248];
        T w22 = J[249];
        T w33 = J[250];
        T w35 = J[251];
        T w37 = T(0);
        T w42 = J[252];
        T w43 = T(0);
        T w44 = J[253];
        T w45 = T(0);
        T w46 = T(0);
        T w47 = T(0);
        T w49 = J[254];
        T w50 = T(0);
        T w51 = T(0);
        T w52 = J[255];
        T w53 = J[256];
        T w54 = T(0);
        T w55 = T(0);
        T w56 = J[257];
        T zt = z[12];
        zt -= w18 * z[5];
        w43 -= w18 * J[58];
        w44 -= w18 * J[59];
        w45 -= w18 * J[60];
        w46 -= w18 * J[61];
        w54 -= w18 * J[62];
        zt -= w21 * z[25];
        w37 -= w21 * J[65];
        w44 -= w21 * J[66];
        w45 -= w21 * J[67];
        w46 -= w21 * J[68];
        w47 -= w21 * J[69];
        w50 -= w21 * J[70];
        w53 -= w21 * J[71];
        zt -= w22 * z[13];
        w44 -= w22 * J[72];
        w45 -= w22 * J[73];
        w46 -= w22 * J[74];
        w47 -= w22 * J[75];
        w56 -= w22 * J[76];
        zt -= w33 * z[1];
        w49 -= w33 * J[125];
        w52 -= w33 * J[126];
        w54 -= w33 * J[127];
        zt -= w35 * z[14];
        w37 -= w35 * J[133];
        w44 -= w35 * J[134];
        w45 -= w35 * J[135];
        w46 -= w35 * J[136];
        w47 -= w35 * J[137];
        w49 -= w35 * J[138];
        w52 -= w35 * J[139];
        w53 -= w35 * J[140];
        w56 -= w35 * J[141];
        zt -= w37 * z[18];
        w42 -= w37 * J[146];
        w44 -= w37 * J[147];
        w45 -= w37 * J[148];
        w46 -= w37 * J[149];
        w47 -= w37 * J[150];
        w49 -= w37 * J[151];
        w50 -= w37 * J[152];
        w51 -= w37 * J[153];
        w52 -= w37 * J[154];
        w53 -= w37 * J[155];
        w54 -= w37 * J[156];
        w56 -= w37 * J[157];
        zt -= w42 * z[27];
        w47 -= w42 * J[186];
        w49 -= w42 * J[187];
        w51 -= w42 * J[188];
        w52 -= w42 * J[189];
        w53 -= w42 * J[190];
        w54 -= w42 * J[191];
        w55 -= w42 * J[192];
        w56 -= w42 * J[193];
        zt -= w43 * z[20];
        w44 -= w43 * J[194];
        w45 -= w43 * J[195];
        w46 -= w43 * J[196];
        w47 -= w43 * J[197];
        w49 -= w43 * J[198];
        w50 -= w43 * J[199];
        w52 -= w43 * J[200];
        w53 -= w43 * J[201];
        w54 -= w43 * J[202];
        w55 -= w43 * J[203];
        w56 -= w43 * J[204];
        T p = w44; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[12] = zt * d;
        J[205] = w45 * d;
        J[206] = w46 * d;
        J[207] = w47 * d;
        J[208] = w49 * d;
        J[209] = w50 * d;
        J[210] = w51 * d;
        J[211] = w52 * d;
        J[212] = w53 * d;
        J[213] = w54 * d;
        J[214] = w55 * d;
        J[215] = w56 * d;
    }
    NT_FENCE();
    {  // row 45: unknown 2
        T w8 = J[258];
        T w26 = J[259];
        T w29 = J[260];
        T w33 = J[261];
        T w38 = J[262];
        T w40 = J[263];
        T w41 = T(0);
        T w42 = J[264];
        T w43 = T(0);
        T w44 = J[265];
        T w45 = J[266];
        T w46 = T(0);
        T w47 = T(0);
        T w49 = T(0);
        T w50 = T(0);
        T w51 = T(0);
        T w52 = J[267];
        T w53 = J[268];
        T w54 = T(0);
        T w55 = T(0);
        T w56 = T(0);
        T zt = z[2];
        zt -= w8 * z[29];
        w41 -= w8 * J[30];
        w52 -= w8 * J[31];
        w53 -= w8 * J[32];
        zt -= w26 * z[42];
        w54 -= w26 * J[80];
        zt -= w29 * z[4];
        w43 -= w29 * J[97];
        w44 -= w29 * J[98];
        w45 -= w29 * J[99];
        w46 -= w29 * J[100];
        w47 -= w29 * J[101];
        w50 -= w29 * J[102];
        w52 -= w29 * J[103];
        w54 -= w29 * J[104];
        w56 -= w29 * J[105];
        zt -= w33 * z[1];
        w49 -= w33 * J[125];
        w52 -= w33 * J[126];
        w54 -= w33 * J[127];
        zt -= w38 * z[16];
        w52 -= w38 * J[158];
        w53 -= w38 * J[159];
        zt -= w40 * z[55];
        w42 -= w40 * J[172];
        w47 -= w40 * J[173];
        w49 -= w40 * J[174];
        w51 -= w40 * J[175];
        w52 -= w40 * J[176];
        w53 -= w40 * J[177];
        w54 -= w40 * J[178];
        zt -= w41 * z[28];
        w47 -= w41 * J[179];
        w49 -= w41 * J[180];
        w52 -= w41 * J[181];
        w53 -= w41 * J[182];
        w54 -= w41 * J[183];
        w55 -= w41 * J[184];
        w56 -= w41 * J[185];
        zt -= w42 * z[27];
        w47 -= w42 * J[186];
        w49 -= w42 * J[187];
        w51 -= w42 * J[188];
        w52 -= w42 * J[189];
        w53 -= w42 * J[190];
        w54 -= w42 * J[191];
        w55 -= w42 * J[192];
        w56 -= w42 * J[193];
        zt -= w43 * z[20];
        w44 -= w43 * J[194];
        w45 -= w43 * J[195];
        w46 -= w43 * J[196];
        w47 -= w43 * J[197];
        w49 -= w43 * J[198];
        w50 -= w43 * J[199];
        w52 -= w43 * J[200];
        w53 -= w43 * J[201];
        w54 -= w43 * J[202];
        w55 -= w43 * J[203];
        w56 -= w43 * J[204];
        zt -= w44 * z[12];
        w45 -= w44 * J[205];
        w46 -= w44 * J[206];
        w47 -= w44 * J[207];
        w49 -= w44 * J[208];
        w50 -= w44 * J[209];
        w51 -= w44 * J[210];
        w52 -= w44 * J[211];
        w53 -= w44 * J[212];
        w54 -= w44 * J[213];
        w55 -= w44 * J[214];
        w56 -= w44 * J[215];
        T p = w45; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[2] = zt * d;
        J[216] = w46 * d;
        J[217] = w47 * d;
        J[218] = w49 * d;
        J[219] = w50 * d;
        J[220] = w51 * d;
        J[221] = w52 * d;
        J[222] = w53 * d;
        J[223] = w54 * d;
        J[224] = w55 * d;
        J[225] = w56 * d;
    }
    NT_FENCE();
    {  // row 46: unknown 48
        T w41 = J[269];
        T w43 = J[270];
        T w44 = T(0);
        T w45 = T(0);
        T w46 = J[271];
        T w47 = J[272];
        T w49 = T(0);
        T w50 = J[273];
        T w51 = T(0);
        T w52 = T(0);
        T w53 = J[274];
        T w54 = J[275];
        T w55 = J[276];
        T w56 = J[277];
        T zt = z[48];
        zt -= w41 * z[28];
        w47 -= w41 * J[179];
        w49 -= w41 * J[180];
        w52 -= w41 * J[181];
        w53 -= w41 * J[182];
        w54 -= w41 * J[183];
        w55 -= w41 * J[184];
        w56 -= w41 * J[185];
        zt -= w43 * z[20];
        w44 -= w43 * J[194];
        w45 -= w43 * J[195];
        w46 -= w43 * J[196];
        w47 -= w43 * J[197];
        w49 -= w43 * J[198];
        w50 -= w43 * J[199];
        w52 -= w43 * J[200];
        w53 -= w43 * J[201];
        w54 -= w43 * J[202];
        w55 -= w43 * J[203];
        w56 -= w43 * J[204];
        zt -= w44 * z[12];
        w45 -= w44 * J[205];
        w46 -= w44 * J[206];
        w47 -= w44 * J[207];
        w49 -= w44 * J[208];
        w50 -= w44 * J[209];
        w51 -= w44 * J[210];
        w52 -= w44 * J[211];
        w53 -= w44 * J[212];
        w54 -= w44 * J[213];
        w55 -= w44 * J[214];
        w56 -= w44 * J[215];
        zt -= w45 * z[2];
        w46 -= w45 * J[216];
        w47 -= w45 * J[217];
        w49 -= w45 * J[218];
        w50 -= w45 * J[219];
        w51 -= w45 * J[220];
        w52 -= w45 * J[221];
        w53 -= w45 * J[222];
        w54 -= w45 * J[223];
        w55 -= w45 * J[224];
        w56 -= w45 * J[225];
        T p = w46; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[48] = zt * d;
        J[226] = w47 * d;
        J[227] = w49 * d;
        J[228] = w50 * d;
        J[229] = w51 * d;
        J[230] = w52 * d;
        J[231] = w53 * d;
        J[232] = w54 * d;
        J[233] = w55 * d;
        J[234] = w56 * d;
    }
    NT_FENCE();
    {  // row 47: unknown 45
        T w40 = J[278];
        T w42 = T(0);
        T w47 = T(1.0);
        T w49 = J[279];
        T w51 = T(0);
        T w52 = J[280];
        T w53 = J[281];
        T w54 = J[282];
        T w55 = J[283];
        T w56 = T(0);
        T zt = z[45];
        zt -= w40 * z[55];
        w42 -= w40 * J[172];
        w47 -= w40 * J[173];
        w49 -= w40 * J[174];
        w51 -= w40 * J[175];
        w52 -= w40 * J[176];
        w53 -= w40 * J[177];
        w54 -= w40 * J[178];
        zt -= w42 * z[27];
        w47 -= w42 * J[186];
        w49 -= w42 * J[187];
        w51 -= w42 * J[188];
        w52 -= w42 * J[189];
        w53 -= w42 * J[190];
        w54 -= w42 * J[191];
        w55 -= w42 * J[192];
        w56 -= w42 * J[193];
        T p = w47; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[45] = zt * d;
        J[235] = w49 * d;
        J[236] = w51 * d;
        J[237] = w52 * d;
        J[238] = w53 * d;
        J[239] = w54 * d;
        J[240] = w55 * d;
        J[241] = w56 * d;
    }
    NT_FENCE();
    {  // row 48: unknown 10
        T w48 = T(1.0);
        T zt = z[10];
        T p = w48; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[10] = zt * d;
    }
    NT_FENCE();
    {  // row 49: unknown 44
        T w33 = J[284];
        T w35 = J[285];
        T w37 = T(0);
        T w41 = J[286];
        T w42 = T(0);
        T w44 = J[287];
        T w45 = J[288];
        T w46 = J[289];
        T w47 = J[290];
        T w49 = T(1.0);
        T w50 = J[291];
        T w51 = T(0);
        T w52 = J[292];
        T w53 = J[293];
        T w54 = J[294];
        T w55 = J[295];
        T w56 = J[296];
        T zt = z[44];
        zt -= w33 * z[1];
        w49 -= w33 * J[125];
        w52 -= w33 * J[126];
        w54 -= w33 * J[127];
        zt -= w35 * z[14];
        w37 -= w35 * J[133];
        w44 -= w35 * J[134];
        w45 -= w35 * J[135];
        w46 -= w35 * J[136];
        w47 -= w35 * J[137];
        w49 -= w35 * J[138];
        w52 -= w35 * J[139];
        w53 -= w35 * J[140];
        w56 -= w35 * J[141];
        zt -= w37 * z[18];
        w42 -= w37 * J[146];
        w44 -= w37 * J[147];
        w45 -= w37 * J[148];
        w46 -= w37 * J[149];
        w47 -= w37 * J[150];
        w49 -= w37 * J[151];
        w50 -= w37 * J[152];
        w51 -= w37 * J[153];
        w52 -= w37 * J[154];
        w53 -= w37 * J[155];
        w54 -= w37 * J[156];
        w56 -= w37 * J[157];
        zt -= w41 * z[28];
        w47 -= w41 * J[179];
        w49 -= w41 * J[180];
        w52 -= w41 * J[181];
        w53 -= w41 * J[182];
        w54 -= w41 * J[183];
        w55 -= w41 * J[184];
        w56 -= w41 * J[185];
        zt -= w42 * z[27];
        w47 -= w42 * J[186];
        w49 -= w42 * J[187];
        w51 -= w42 * J[188];
        w52 -= w42 * J[189];
        w53 -= w42 * J[190];
        w54 -= w42 * J[191];
        w55 -= w42 * J[192];
        w56 -= w42 * J[193];
        zt -= w44 * z[12];
        w45 -= w44 * J[205];
        w46 -= w44 * J[206];
        w47 -= w44 * J[207];
        w49 -= w44 * J[208];
        w50 -= w44 * J[209];
        w51 -= w44 * J[210];
        w52 -= w44 * J[211];
        w53 -= w44 * J[212];
        w54 -= w44 * J[213];
        w55 -= w44 * J[214];
        w56 -= w44 * J[215];
        zt -= w45 * z[2];
        w46 -= w45 * J[216];
        w47 -= w45 * J[217];
        w49 -= w45 * J[218];
        w50 -= w45 * J[219];
        w51 -= w45 * J[220];
        w52 -= w45 * J[221];
        w53 -= w45 * J[222];
        w54 -= w45 * J[223];
        w55 -= w45 * J[224];
        w56 -= w45 * J[225];
        zt -= w46 * z[48];
        w47 -= w46 * J[226];
        w49 -= w46 * J[227];
        w50 -= w46 * J[228];
        w51 -= w46 * J[229];
        w52 -= w46 * J[230];
        w53 -= w46 * J[231];
        w54 -= w46 * J[232];
        w55 -= w46 * J[233];
        w56 -= w46 * J[234];
        zt -= w47 * z[45];
        w49 -= w47 * J[235];
        w51 -= w47 * J[236];
        w52 -= w47 * J[237];
        w53 -= w47 * J[238];
        w54 -= w47 * J[239];
        w55 -= w47 * J[240];
        w56 -= w47 * J[241];
        T p = w49; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[44] = zt * d;
        J[242] = w50 * d;
        J[243] = w51 * d;
        J[244] = w52 * d;
        J[245] = w53 * d;
        J[246] = w54 * d;
        J[247] = w55 * d;
        J[248] = w56 * d;
    }
    NT_FENCE();
    {  // row 50: unknown 53
        T w39 = J[297];
        T w42 = J[298];
        T w44 = T(0);
        T w45 = T(0);
        T w46 = J[299];
        T w47 = J[300];
        T w49 = T(0);
        T w50 = J[301];
        T w51 = T(0);
        T w52 = J[302];
        T w53 = J[303];
        T w54 = J[304];
        T w55 = J[305];
        T w56 = J[306];
        T zt = z[53];
        zt -= w39 * z[23];
        w42 -= w39 * J[160];
        w44 -= w39 * J[161];
        w45 -= w39 * J[162];
        w46 -= w39 * J[163];
        w47 -= w39 * J[164];
        w49 -= w39 * J[165];
        w50 -= w39 * J[166];
        w51 -= w39 * J[167];
        w52 -= w39 * J[168];
        w53 -= w39 * J[169];
        w54 -= w39 * J[170];
        w56 -= w39 * J[171];
        zt -= w42 * z[27];
        w47 -= w42 * J[186];
        w49 -= w42 * J[187];
        w51 -= w42 * J[188];
        w52 -= w42 * J[189];
        w53 -= w42 * J[190];
        w54 -= w42 * J[191];
        w55 -= w42 * J[192];
        w56 -= w42 * J[193];
        zt -= w44 * z[12];
        w45 -= w44 * J[205];
        w46 -= w44 * J[206];
        w47 -= w44 * J[207];
        w49 -= w44 * J[208];
        w50 -= w44 * J[209];
        w51 -= w44 * J[210];
        w52 -= w44 * J[211];
        w53 -= w44 * J[212];
        w54 -= w44 * J[213];
        w55 -= w44 * J[214];
        w56 -= w44 * J[215];
        zt -= w45 * z[2];
        w46 -= w45 * J[216];
        w47 -= w45 * J[217];
        w49 -= w45 * J[218];
        w50 -= w45 * J[219];
        w51 -= w45 * J[220];
        w52 -= w45 * J[221];
        w53 -= w45 * J[222];
        w54 -= w45 * J[223];
        w55 -= w45 * J[224];
        w56 -= w45 * J[225];
        zt -= w46 * z[48];
        w47 -= w46 * J[226];
        w49 -= w46 * J[227];
        w50 -= w46 * J[228];
        w51 -= w46 * J[229];
        w52 -= w46 * J[230];
        w53 -= w46 * J[231];
        w54 -= w46 * J[232];
        w55 -= w46 * J[233];
        w56 -= w46 * J[234];
        zt -= w47 * z[45];
        w49 -= w47 * J[235];
        w51 -= w47 * J[236];
        w52 -= w47 * J[237];
        w53 -= w47 * J[238];
        w54 -= w47 * J[239];
        w55 -= w47 * J[240];
        w56 -= w47 * J[241];
        zt -= w49 * z[44];
        w50 -= w49 * J[242];
        w51 -= w49 * J[243];
        w52 -= w49 * J[244];
        w53 -= w49 * J[245];
        w54 -= w49 * J[246];
        w55 -= w49 * J[247];
        w56 -= w49 * J[248];
        T p = w50; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[53] = zt * d;
        J[249] = w51 * d;
        J[250] = w52 * d;
        J[251] = w53 * d;
        J[252] = w54 * d;
        J[253] = w55 * d;
        J[254] = w56 * d;
    }
    NT_FENCE();
    {  // row 51: unknown 50
        T w42 = J[307];
        T w46 = J[308];
        T w47 = J[309];
        T w49 = T(0);
        T w50 = J[310];
        T w51 = T(1.0);
        T w52 = J[311];
        T w53 = J[312];
        T w54 = J[313];
        T w55 = J[314];
        T w56 = J[315];
        T zt = z[50];
        zt -= w42 * z[27];
        w47 -= w42 * J[186];
        w49 -= w42 * J[187];
        w51 -= w42 * J[188];
        w52 -= w42 * J[189];
        w53 -= w42 * J[190];
        w54 -= w42 * J[191];
        w55 -= w42 * J[192];
        w56 -= w42 * J[193];
        zt -= w46 * z[48];
        w47 -= w46 * J[226];
        w49 -= w46 * J[227];
        w50 -= w46 * J[228];
        w51 -= w46 * J[229];
        w52 -= w46 * J[230];
        w53 -= w46 * J[231];
        w54 -= w46 * J[232];
        w55 -= w46 * J[233];
        w56 -= w46 * J[234];
        zt -= w47 * z[45];
        w49 -= w47 * J[235];
        w51 -= w47 * J[236];
        w52 -= w47 * J[237];
        w53 -= w47 * J[238];
        w54 -= w47 * J[239];
        w55 -= w47 * J[240];
        w56 -= w47 * J[241];
        zt -= w49 * z[44];
        w50 -= w49 * J[242];
        w51 -= w49 * J[243];
        w52 -= w49 * J[244];
        w53 -= w49 * J[245];
        w54 -= w49 * J[246];
        w55 -= w49 * J[247];
        w56 -= w49 * J[248];
        zt -= w50 * z[53];
        w51 -= w50 * J[249];
        w52 -= w50 * J[250];
        w53 -= w50 * J[251];
        w54 -= w50 * J[252];
        w55 -= w50 * J[253];
        w56 -= w50 * J[254];
        T p = w51; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[50] = zt * d;
        J[255] = w52 * d;
        J[256] = w53 * d;
        J[257] = w54 * d;
        J[258] = w55 * d;
        J[259] = w56 * d;
    }
    NT_FENCE();
    {  // row 52: unknown 43
        T w8 = J[316];
        T w21 = J[317];
        T w26 = J[318];
        T w29 = J[319];
        T w32 = J[320];
        T w33 = J[321];
        T w34 = J[322];
        T w35 = J[323];
        T w36 = J[324];
        T w37 = J[325];
        T w38 = J[326];
        T w40 = J[327];
        T w41 = J[328];
        T w42 = J[329];
        T w43 = T(0);
        T w44 = J[330];
        T w45 = J[331];
        T w46 = J[332];
        T w47 = J[333];
        T w49 = J[334];
        T w50 = J[335];
        T w51 = J[336];
        T w52 = J[337];
        T w53 = J[338];
        T w54 = J[339];
        T w55 = J[340];
        T w56 = J[341];
        T zt = z[43];
        zt -= w8 * z[29];
        w41 -= w8 * J[30];
        w52 -= w8 * J[31];
        w53 -= w8 * J[32];
        zt -= w21 * z[25];
        w37 -= w21 * J[65];
        w44 -= w21 * J[66];
        w45 -= w21 * J[67];
        w46 -= w21 * J[68];
        w47 -= w21 * J[69];
        w50 -= w21 * J[70];
        w53 -= w21 * J[71];
        zt -= w26 * z[42];
        w54 -= w26 * J[80];
        zt -= w29 * z[4];
        w43 -= w29 * J[97];
        w44 -= w29 * J[98];
        w45 -= w29 * J[99];
        w46 -= w29 * J[100];
        w47 -= w29 * J[101];
        w50 -= w29 * J[102];
        w52 -= w29 * J[103];
        w54 -= w29 * J[104];
        w56 -= w29 * J[105];
        zt -= w32 * z[21];
        w46 -= w32 * J[122];
        w52 -= w32 * J[123];
        w53 -= w32 * J[124];
        zt -= w33 * z[1];
        w49 -= w33 * J[125];
        w52 -= w33 * J[126];
        w54 -= w33 * J[127];
        zt -= w34 * z[8];
        w42 -= w34 * J[128];
        w47 -= w34 * J[129];
        w49 -= w34 * J[130];
        w51 -= w34 * J[131];
        w52 -= w34 * J[132];
        zt -= w35 * z[14];
        w37 -= w35 * J[133];
        w44 -= w35 * J[134];
        w45 -= w35 * J[135];
        w46 -= w35 * J[136];
        w47 -= w35 * J[137];
        w49 -= w35 * J[138];
        w52 -= w35 * J[139];
        w53 -= w35 * J[140];
        w56 -= w35 * J[141];
        zt -= w36 * z[56];
        w47 -= w36 * J[142];
        w49 -= w36 * J[143];
        w52 -= w36 * J[144];
        w54 -= w36 * J[145];
        zt -= w37 * z[18];
        w42 -= w37 * J[146];
        w44 -= w37 * J[147];
        w45 -= w37 * J[148];
        w46 -= w37 * J[149];
        w47 -= w37 * J[150];
        w49 -= w37 * J[151];
        w50 -= w37 * J[152];
        w51 -= w37 * J[153];
        w52 -= w37 * J[154];
        w53 -= w37 * J[155];
        w54 -= w37 * J[156];
        w56 -= w37 * J[157];
        zt -= w38 * z[16];
        w52 -= w38 * J[158];
        w53 -= w38 * J[159];
        zt -= w40 * z[55];
        w42 -= w40 * J[172];
        w47 -= w40 * J[173];
        w49 -= w40 * J[174];
        w51 -= w40 * J[175];
        w52 -= w40 * J[176];
        w53 -= w40 * J[177];
        w54 -= w40 * J[178];
        zt -= w41 * z[28];
        w47 -= w41 * J[179];
        w49 -= w41 * J[180];
        w52 -= w41 * J[181];
        w53 -= w41 * J[182];
        w54 -= w41 * J[183];
        w55 -= w41 * J[184];
        w56 -= w41 * J[185];
        zt -= w42 * z[27];
        w47 -= w42 * J[186];
        w49 -= w42 * J[187];
        w51 -= w42 * J[188];
        w52 -= w42 * J[189];
        w53 -= w42 * J[190];
        w54 -= w42 * J[191];
        w55 -= w42 * J[192];
        w56 -= w42 * J[193];
        zt -= w43 * z[20];
        w44 -= w43 * J[194];
        w45 -= w43 * J[195];
        w46 -= w43 * J[196];
        w47 -= w43 * J[197];
        w49 -= w43 * J[198];
        w50 -= w43 * J[199];
        w52 -= w43 * J[200];
        w53 -= w43 * J[201];
        w54 -= w43 * J[202];
        w55 -= w43 * J[203];
        w56 -= w43 * J[204];
        zt -= w44 * z[12];
        w45 -= w44 * J[205];
        w46 -= w44 * J[206];
        w47 -= w44 * J[207];
        w49 -= w44 * J[208];
        w50 -= w44 * J[209];
        w51 -= w44 * J[210];
        w52 -= w44 * J[211];
        w53 -= w44 * J[212];
        w54 -= w44 * J[213];
        w55 -= w44 * J[214];
        w56 -= w44 * J[215];
        zt -= w45 * z[2];
        w46 -= w45 * J[216];
        w47 -= w45 * J[217];
        w49 -= w45 * J[218];
        w50 -= w45 * J[219];
        w51 -= w45 * J[220];
        w52 -= w45 * J[221];
        w53 -= w45 * J[222];
        w54 -= w45 * J[223];
        w55 -= w45 * J[224];
        w56 -= w45 * J[225];
        zt -= w46 * z[48];
        w47 -= w46 * J[226];
        w49 -= w46 * J[227];
        w50 -= w46 * J[228];
        w51 -= w46 * J[229];
        w52 -= w46 * J[230];
        w53 -= w46 * J[231];
        w54 -= w46 * J[232];
        w55 -= w46 * J[233];
        w56 -= w46 * J[234];
        zt -= w47 * z[45];
        w49 -= w47 * J[235];
        w51 -= w47 * J[236];
        w52 -= w47 * J[237];
        w53 -= w47 * J[238];
        w54 -= w47 * J[239];
        w55 -= w47 * J[240];
        w56 -= w47 * J[241];
        zt -= w49 * z[44];
        w50 -= w49 * J[242];
        w51 -= w49 * J[243];
        w52 -= w49 * J[244];
        w53 -= w49 * J[245];
        w54 -= w49 * J[246];
        w55 -= w49 * J[247];
        w56 -= w49 * J[248];
        zt -= w50 * z[53];
        w51 -= w50 * J[249];
        w52 -= w50 * J[250];
        w53 -= w50 * J[251];
        w54 -= w50 * J[252];
        w55 -= w50 * J[253];
        w56 -= w50 * J[254];
        zt -= w51 * z[50];
        w52 -= w51 * J[255];
        w53 -= w51 * J[256];
        w54 -= w51 * J[257];
        w55 -= w51 * J[258];
        w56 -= w51 * J[259];
        T p = w52; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[43] = zt * d;
        J[260] = w53 * d;
        J[261] = w54 * d;
        J[262] = w55 * d;
        J[263] = w56 * d;
    }
    NT_FENCE();
    {  // row 53: unknown 47
        T w34 = J[342];
        T w38 = J[343];
        T w40 = J[344];
        T w42 = J[345];
        T w47 = J[346];
        T w49 = J[347];
        T w50 = J[348];
        T w51 = J[349];
        T w52 = J[350];
        T w53 = J[351];
        T w54 = J[352];
        T w55 = J[353];
        T w56 = J[354];
        T zt = z[47];
        zt -= w34 * z[8];
        w42 -= w34 * J[128];
        w47 -= w34 * J[129];
        w49 -= w34 * J[130];
        w51 -= w34 * J[131];
        w52 -= w34 * J[132];
        zt -= w38 * z[16];
        w52 -= w38 * J[158];
        w53 -= w38 * J[159];
        zt -= w40 * z[55];
        w42 -= w40 * J[172];
        w47 -= w40 * J[173];
        w49 -= w40 * J[174];
        w51 -= w40 * J[175];
        w52 -= w40 * J[176];
        w53 -= w40 * J[177];
        w54 -= w40 * J[178];
        zt -= w42 * z[27];
        w47 -= w42 * J[186];
        w49 -= w42 * J[187];
        w51 -= w42 * J[188];
        w52 -= w42 * J[189];
        w53 -= w42 * J[190];
        w54 -= w42 * J[191];
        w55 -= w42 * J[192];
        w56 -= w42 * J[193];
        zt -= w47 * z[45];
        w49 -= w47 * J[235];
        w51 -= w47 * J[236];
        w52 -= w47 * J[237];
        w53 -= w47 * J[238];
        w54 -= w47 * J[239];
        w55 -= w47 * J[240];
        w56 -= w47 * J[241];
        zt -= w49 * z[44];
        w50 -= w49 * J[242];
        w51 -= w49 * J[243];
        w52 -= w49 * J[244];
        w53 -= w49 * J[245];
        w54 -= w49 * J[246];
        w55 -= w49 * J[247];
        w56 -= w49 * J[248];
        zt -= w50 * z[53];
        w51 -= w50 * J[249];
        w52 -= w50 * J[250];
        w53 -= w50 * J[251];
        w54 -= w50 * J[252];
        w55 -= w50 * J[253];
        w56 -= w50 * J[254];
        zt -= w51 * z[50];
        w52 -= w51 * J[255];
        w53 -= w51 * J[256];
        w54 -= w51 * J[257];
        w55 -= w51 * J[258];
        w56 -= w51 * J[259];
        zt -= w52 * z[43];
        w53 -= w52 * J[260];
        w54 -= w52 * J[261];
        w55 -= w52 * J[262];
        w56 -= w52 * J[263];
        T p = w53; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[47] = zt * d;
        J[264] = w54 * d;
        J[265] = w55 * d;
        J[266] = w56 * d;
    }
    NT_FENCE();
    {  // row 54: unknown 46
        T w28 = J[355];
        T w35 = T(0);
        T w37 = T(0);
        T w40 = J[356];
        T w41 = T(0);
        T w42 = T(0);
        T w44 = T(0);
        T w45 = T(0);
        T w46 = T(0);
        T w47 = T(0);
        T w49 = J[357];
        T w50 = T(0);
        T w51 = T(0);
        T w52 = J[358];
        T w53 = J[359];
        T w54 = T(1.0);
        T w55 = J[360];
        T w56 = T(0);
        T zt = z[46];
        zt -= w28 * z[7];
        w35 -= w28 * J[83];
        w37 -= w28 * J[84];
        w40 -= w28 * J[85];
        w41 -= w28 * J[86];
        w44 -= w28 * J[87];
        w45 -= w28 * J[88];
        w46 -= w28 * J[89];
        w47 -= w28 * J[90];
        w50 -= w28 * J[91];
        w52 -= w28 * J[92];
        w53 -= w28 * J[93];
        w54 -= w28 * J[94];
        w55 -= w28 * J[95];
        w56 -= w28 * J[96];
        zt -= w35 * z[14];
        w37 -= w35 * J[133];
        w44 -= w35 * J[134];
        w45 -= w35 * J[135];
        w46 -= w35 * J[136];
        w47 -= w35 * J[137];
        w49 -= w35 * J[138];
        w52 -= w35 * J[139];
        w53 -= w35 * J[140];
        w56 -= w35 * J[141];
        zt -= w37 * z[18];
        w42 -= w37 * J[146];
        w44 -= w37 * J[147];
        w45 -= w37 * J[148];
        w46 -= w37 * J[149];
        w47 -= w37 * J[150];
        w49 -= w37 * J[151];
        w50 -= w37 * J[152];
        w51 -= w37 * J[153];
        w52 -= w37 * J[154];
        w53 -= w37 * J[155];
        w54 -= w37 * J[156];
        w56 -= w37 * J[157];
        zt -= w40 * z[55];
        w42 -= w40 * J[172];
        w47 -= w40 * J[173];
        w49 -= w40 * J[174];
        w51 -= w40 * J[175];
        w52 -= w40 * J[176];
        w53 -= w40 * J[177];
        w54 -= w40 * J[178];
        zt -= w41 * z[28];
        w47 -= w41 * J[179];
        w49 -= w41 * J[180];
        w52 -= w41 * J[181];
        w53 -= w41 * J[182];
        w54 -= w41 * J[183];
        w55 -= w41 * J[184];
        w56 -= w41 * J[185];
        zt -= w42 * z[27];
        w47 -= w42 * J[186];
        w49 -= w42 * J[187];
        w51 -= w42 * J[188];
        w52 -= w42 * J[189];
        w53 -= w42 * J[190];
        w54 -= w42 * J[191];
        w55 -= w42 * J[192];
        w56 -= w42 * J[193];
        zt -= w44 * z[12];
        w45 -= w44 * J[205];
        w46 -= w44 * J[206];
        w47 -= w44 * J[207];
        w49 -= w44 * J[208];
        w50 -= w44 * J[209];
        w51 -= w44 * J[210];
        w52 -= w44 * J[211];
        w53 -= w44 * J[212];
        w54 -= w44 * J[213];
        w55 -= w44 * J[214];
        w56 -= w44 * J[215];
        zt -= w45 * z[2];
        w46 -= w45 * J[216];
        w47 -= w45 * J[217];
        w49 -= w45 * J[218];
        w50 -= w45 * J[219];
        w51 -= w45 * J[220];
        w52 -= w45 * J[221];
        w53 -= w45 * J[222];
        w54 -= w45 * J[223];
        w55 -= w45 * J[224];
        w56 -= w45 * J[225];
        zt -= w46 * z[48];
        w47 -= w46 * J[226];
        w49 -= w46 * J[227];
        w50 -= w46 * J[228];
        w51 -= w46 * J[229];
        w52 -= w46 * J[230];
        w53 -= w46 * J[231];
        w54 -= w46 * J[232];
        w55 -= w46 * J[233];
        w56 -= w46 * J[234];
        zt -= w47 * z[45];
        w49 -= w47 * J[235];
        w51 -= w47 * J[236];
        w52 -= w47 * J[237];
        w53 -= w47 * J[238];
        w54 -= w47 * J[239];
        w55 -= w47 * J[240];
        w56 -= w47 * J[241];
        zt -= w49 * z[44];
        w50 -= w49 * J[242];
        w51 -= w49 * J[243];
        w52 -= w49 * J[244];
        w53 -= w49 * J[245];
        w54 -= w49 * J[246];
        w55 -= w49 * J[247];
        w56 -= w49 * J[248];
        zt -= w50 * z[53];
        w51 -= w50 * J[249];
        w52 -= w50 * J[250];
        w53 -= w50 * J[251];
        w54 -= w50 * J[252];
        w55 -= w50 * J[253];
        w56 -= w50 * J[254];
        zt -= w51 * z[50];
        w52 -= w51 * J[255];
        w53 -= w51 * J[256];
        w54 -= w51 * J[257];
        w55 -= w51 * J[258];
        w56 -= w51 * J[259];
        zt -= w52 * z[43];
        w53 -= w52 * J[260];
        w54 -= w52 * J[261];
        w55 -= w52 * J[262];
        w56 -= w52 * J[263];
        zt -= w53 * z[47];
        w54 -= w53 * J[264];
        w55 -= w53 * J[265];
        w56 -= w53 * J[266];
        T p = w54; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[46] = zt * d;
        J[267] = w55 * d;
        J[268] = w56 * d;
    }
    NT_FENCE();
    {  // row 55: unknown 49
        T w41 = J[361];
        T w46 = J[362];
        T w47 = J[363];
        T w49 = T(0);
        T w50 = J[364];
        T w51 = T(0);
        T w52 = T(0);
        T w53 = J[365];
        T w54 = J[366];
        T w55 = T(1.0);
        T w56 = J[367];
        T zt = z[49];
        zt -= w41 * z[28];
        w47 -= w41 * J[179];
        w49 -= w41 * J[180];
        w52 -= w41 * J[181];
        w53 -= w41 * J[182];
        w54 -= w41 * J[183];
        w55 -= w41 * J[184];
        w56 -= w41 * J[185];
        zt -= w46 * z[48];
        w47 -= w46 * J[226];
        w49 -= w46 * J[227];
        w50 -= w46 * J[228];
        w51 -= w46 * J[229];
        w52 -= w46 * J[230];
        w53 -= w46 * J[231];
        w54 -= w46 * J[232];
        w55 -= w46 * J[233];
        w56 -= w46 * J[234];
        zt -= w47 * z[45];
        w49 -= w47 * J[235];
        w51 -= w47 * J[236];
        w52 -= w47 * J[237];
        w53 -= w47 * J[238];
        w54 -= w47 * J[239];
        w55 -= w47 * J[240];
        w56 -= w47 * J[241];
        zt -= w49 * z[44];
        w50 -= w49 * J[242];
        w51 -= w49 * J[243];
        w52 -= w49 * J[244];
        w53 -= w49 * J[245];
        w54 -= w49 * J[246];
        w55 -= w49 * J[247];
        w56 -= w49 * J[248];
        zt -= w50 * z[53];
        w51 -= w50 * J[249];
        w52 -= w50 * J[250];
        w53 -= w50 * J[251];
        w54 -= w50 * J[252];
        w55 -= w50 * J[253];
        w56 -= w50 * J[254];
        zt -= w51 * z[50];
        w52 -= w51 * J[255];
        w53 -= w51 * J[256];
        w54 -= w51 * J[257];
        w55 -= w51 * J[258];
        w56 -= w51 * J[259];
        zt -= w52 * z[43];
        w53 -= w52 * J[260];
        w54 -= w52 * J[261];
        w55 -= w52 * J[262];
        w56 -= w52 * J[263];
        zt -= w53 * z[47];
        w54 -= w53 * J[264];
        w55 -= w53 * J[265];
        w56 -= w53 * J[266];
        zt -= w54 * z[46];
        w55 -= w54 * J[267];
        w56 -= w54 * J[268];
        T p = w55; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[49] = zt * d;
        J[269] = w56 * d;
    }
    NT_FENCE();
    {  // row 56: unknown 52
        T w31 = J[368];
        T w33 = J[369];
        T w35 = J[370];
        T w37 = T(0);
        T w41 = J[371];
        T w42 = T(0);
        T w43 = T(0);
        T w44 = J[372];
        T w45 = J[373];
        T w46 = J[374];
        T w47 = J[375];
        T w49 = T(0);
        T w50 = J[376];
        T w51 = T(0);
        T w52 = J[377];
        T w53 = J[378];
        T w54 = J[379];
        T w55 = J[380];
        T w56 = J[381];
        T zt = z[52];
        zt -= w31 * z[22];
        w33 -= w31 * J[107];
        w35 -= w31 * J[108];
        w37 -= w31 * J[109];
        w42 -= w31 * J[110];
        w43 -= w31 * J[111];
        w44 -= w31 * J[112];
        w45 -= w31 * J[113];
        w46 -= w31 * J[114];
        w47 -= w31 * J[115];
        w49 -= w31 * J[116];
        w50 -= w31 * J[117];
        w52 -= w31 * J[118];
        w53 -= w31 * J[119];
        w54 -= w31 * J[120];
        w56 -= w31 * J[121];
        zt -= w33 * z[1];
        w49 -= w33 * J[125];
        w52 -= w33 * J[126];
        w54 -= w33 * J[127];
        zt -= w35 * z[14];
        w37 -= w35 * J[133];
        w44 -= w35 * J[134];
        w45 -= w35 * J[135];
        w46 -= w35 * J[136];
        w47 -= w35 * J[137];
        w49 -= w35 * J[138];
        w52 -= w35 * J[139];
        w53 -= w35 * J[140];
        w56 -= w35 * J[141];
        zt -= w37 * z[18];
        w42 -= w37 * J[146];
        w44 -= w37 * J[147];
        w45 -= w37 * J[148];
        w46 -= w37 * J[149];
        w47 -= w37 * J[150];
        w49 -= w37 * J[151];
        w50 -= w37 * J[152];
        w51 -= w37 * J[153];
        w52 -= w37 * J[154];
        w53 -= w37 * J[155];
        w54 -= w37 * J[156];
        w56 -= w37 * J[157];
        zt -= w41 * z[28];
        w47 -= w41 * J[179];
        w49 -= w41 * J[180];
        w52 -= w41 * J[181];
        w53 -= w41 * J[182];
        w54 -= w41 * J[183];
        w55 -= w41 * J[184];
        w56 -= w41 * J[185];
        zt -= w42 * z[27];
        w47 -= w42 * J[186];
        w49 -= w42 * J[187];
        w51 -= w42 * J[188];
        w52 -= w42 * J[189];
        w53 -= w42 * J[190];
        w54 -= w42 * J[191];
        w55 -= w42 * J[192];
        w56 -= w42 * J[193];
        zt -= w43 * z[20];
        w44 -= w43 * J[194];
        w45 -= w43 * J[195];
        w46 -= w43 * J[196];
        w47 -= w43 * J[197];
        w49 -= w43 * J[198];
        w50 -= w43 * J[199];
        w52 -= w43 * J[200];
        w53 -= w43 * J[201];
        w54 -= w43 * J[202];
        w55 -= w43 * J[203];
        w56 -= w43 * J[204];
        zt -= w44 * z[12];
        w45 -= w44 * J[205];
        w46 -= w44 * J[206];
        w47 -= w44 * J[207];
        w49 -= w44 * J[208];
        w50 -= w44 * J[209];
        w51 -= w44 * J[210];
        w52 -= w44 * J[211];
        w53 -= w44 * J[212];
        w54 -= w44 * J[213];
        w55 -= w44 * J[214];
        w56 -= w44 * J[215];
        zt -= w45 * z[2];
        w46 -= w45 * J[216];
        w47 -= w45 * J[217];
        w49 -= w45 * J[218];
        w50 -= w45 * J[219];
        w51 -= w45 * J[220];
        w52 -= w45 * J[221];
        w53 -= w45 * J[222];
        w54 -= w45 * J[223];
        w55 -= w45 * J[224];
        w56 -= w45 * J[225];
        zt -= w46 * z[48];
        w47 -= w46 * J[226];
        w49 -= w46 * J[227];
        w50 -= w46 * J[228];
        w51 -= w46 * J[229];
        w52 -= w46 * J[230];
        w53 -= w46 * J[231];
        w54 -= w46 * J[232];
        w55 -= w46 * J[233];
        w56 -= w46 * J[234];
        zt -= w47 * z[45];
        w49 -= w47 * J[235];
        w51 -= w47 * J[236];
        w52 -= w47 * J[237];
        w53 -= w47 * J[238];
        w54 -= w47 * J[239];
        w55 -= w47 * J[240];
        w56 -= w47 * J[241];
        zt -= w49 * z[44];
        w50 -= w49 * J[242];
        w51 -= w49 * J[243];
        w52 -= w49 * J[244];
        w53 -= w49 * J[245];
        w54 -= w49 * J[246];
        w55 -= w49 * J[247];
        w56 -= w49 * J[248];
        zt -= w50 * z[53];
        w51 -= w50 * J[249];
        w52 -= w50 * J[250];
        w53 -= w50 * J[251];
        w54 -= w50 * J[252];
        w55 -= w50 * J[253];
        w56 -= w50 * J[254];
        zt -= w51 * z[50];
        w52 -= w51 * J[255];
        w53 -= w51 * J[256];
        w54 -= w51 * J[257];
        w55 -= w51 * J[258];
        w56 -= w51 * J[259];
        zt -= w52 * z[43];
        w53 -= w52 * J[260];
        w54 -= w52 * J[261];
        w55 -= w52 * J[262];
        w56 -= w52 * J[263];
        zt -= w53 * z[47];
        w54 -= w53 * J[264];
        w55 -= w53 * J[265];
        w56 -= w53 * J[266];
        zt -= w54 * z[46];
        w55 -= w54 * J[267];
        w56 -= w54 * J[268];
        zt -= w55 * z[49];
        w56 -= w55 * J[269];
        T p = w56; if (!(fabs(p) > tiny)) p = (p < T(0)) ? -tiny : tiny;
        const T d = nt_rcp<T>(p);
        z[52] = zt * d;
    }
    NT_FENCE();
    z[49] = z[49] - J[269] * z[52];
    NT_FENCE();
    z[46] = z[46] - J[267] * z[49] - J[268] * z[52];
    NT_FENCE();
    z[47] = z[47] - J[264] * z[46] - J[265] * z[49] - J[266] * z[52];
    NT_FENCE();
    z[43] = z[43] - J[260] * z[47] - J[261] * z[46] - J[262] * z[49] - J[263] * z[52];
    NT_FENCE();
    z[50] = z[50] - J[255] * z[43] - J[256] * z[47] - J[257] * z[46] - J[258] * z[49] - J[259] * z[52];
    NT_FENCE();
    z[53] = z[53] - J[249] * z[50] - J[250] * z[43] - J[251] * z[47] - J[252] * z[46] - J[253] * z[49] - J[254] * z[52];
    NT_FENCE();
    z[44] = z[44] - J[242] * z[53] - J[243] * z[50] - J[244] * z[43] - J[245] * z[47] - J[246] * z[46] - J[247] * z[49] - J[248] * z[52];
    NT_FENCE();
    z[45] = z[45] - J[235] * z[44] - J[236] * z[50] - J[237] * z[43] - J[238] * z[47] - J[239] * z[46] - J[240] * z[49] - J[241] * z[52];
    NT_FENCE();
    z[48] = z[48] - J[226] * z[45] - J[227] * z[44] - J[228] * z[53] - J[229] * z[50] - J[230] * z[43] - J[231] * z[47] - J[232] * z[46] - J[233] * z[49] - J[234] * z[52];
    NT_FENCE();
    z[2] = z[2] - J[216] * z[48] - J[217] * z[45] - J[218] * z[44] - J[219] * z[53] - J[220] * z[50] - J[221] * z[43] - J[222] * z[47] - J[223] * z[46] - J[224] * z[49] - J[225] * z[52];
    NT_FENCE();
    z[12] = z[12] - J[205] * z[2] - J[206] * z[48] - J[207] * z[45] - J[208] * z[44] - J[209] * z[53] - J[210] * z[50] - J[211] * z[43] - J[212] * z[47] - J[213] * z[46] - J[214] * z[49] - J[215] * z[52];
    NT_FENCE();
    z[20] = z[20] - J[194] * z[12] - J[195] * z[2] - J[196] * z[48] - J[197] * z[45] - J[198] * z[44] - J[199] * z[53] - J[200] * z[43] - J[201] * z[47] - J[202] * z[46] - J[203] * z[49] - J[204] * z[52];
    NT_FENCE();
    z[27] = z[27] - J[186] * z[45] - J[187] * z[44] - J[188] * z[50] - J[189] * z[43] - J[190] * z[47] - J[191] * z[46] - J[192] * z[49] - J[193] * z[52];
    NT_FENCE();
    z[28] = z[28] - J[179] * z[45] - J[180] * z[44] - J[181] * z[43] - J[182] * z[47] - J[183] * z[46] - J[184] * z[49] - J[185] * z[52];
    NT_FENCE();
    z[55] = z[55] - J[172] * z[27] - J[173] * z[45] - J[174] * z[44] - J[175] * z[50] - J[176] * z[43] - J[177] * z[47] - J[178] * z[46];
    NT_FENCE();
    z[23] = z[23] - J[160] * z[27] - J[161] * z[12] - J[162] * z[2] - J[163] * z[48] - J[164] * z[45] - J[165] * z[44] - J[166] * z[53] - J[167] * z[50] - J[168] * z[43] - J[169] * z[47] - J[170] * z[46] - J[171] * z[52];
    NT_FENCE();
    z[16] = z[16] - J[158] * z[43] - J[159] * z[47];
    NT_FENCE();
    z[18] = z[18] - J[146] * z[27] - J[147] * z[12] - J[148] * z[2] - J[149] * z[48] - J[150] * z[45] - J[151] * z[44] - J[152] * z[53] - J[153] * z[50] - J[154] * z[43] - J[155] * z[47] - J[156] * z[46] - J[157] * z[52];
    NT_FENCE();
    z[56] = z[56] - J[142] * z[45] - J[143] * z[44] - J[144] * z[43] - J[145] * z[46];
    NT_FENCE();
    z[14] = z[14] - J[133] * z[18] - J[134] * z[12] - J[135] * z[2] - J[136] * z[48] - J[137] * z[45] - J[138] * z[44] - J[139] * z[43] - J[140] * z[47] - J[141] * z[52];
    NT_FENCE();
    z[8] = z[8] - J[128] * z[27] - J[129] * z[45] - J[130] * z[44] - J[131] * z[50] - J[132] * z[43];
    NT_FENCE();
    z[1] = z[1] - J[125] * z[44] - J[126] * z[43] - J[127] * z[46];
    NT_FENCE();
    z[21] = z[21] - J[122] * z[48] - J[123] * z[43] - J[124] * z[47];
    NT_FENCE();
    z[22] = z[22] - J[107] * z[1] - J[108] * z[14] - J[109] * z[18] - J[110] * z[27] - J[111] * z[20] - J[112] * z[12] - J[113] * z[2] - J[114] * z[48] - J[115] * z[45] - J[116] * z[44] - J[117] * z[53] - J[118] * z[43] - J[119] * z[47] - J[120] * z[46] - J[121] * z[52];
    NT_FENCE();
    z[41] = z[41] - J[106] * z[43];
    NT_FENCE();
    z[4] = z[4] - J[97] * z[20] - J[98] * z[12] - J[99] * z[2] - J[100] * z[48] - J[101] * z[45] - J[102] * z[53] - J[103] * z[43] - J[104] * z[46] - J[105] * z[52];
    NT_FENCE();
    z[7] = z[7] - J[83] * z[14] - J[84] * z[18] - J[85] * z[55] - J[86] * z[28] - J[87] * z[12] - J[88] * z[2] - J[89] * z[48] - J[90] * z[45] - J[91] * z[53] - J[92] * z[43] - J[93] * z[47] - J[94] * z[46] - J[95] * z[49] - J[96] * z[52];
    NT_FENCE();
    z[9] = z[9] - J[81] * z[53] - J[82] * z[52];
    NT_FENCE();
    z[42] = z[42] - J[80] * z[46];
    NT_FENCE();
    z[24] = z[24] - J[79] * z[52];
    NT_FENCE();
    z[30] = z[30] - J[78] * z[42];
    NT_FENCE();
    z[34] = z[34] - J[77] * z[43];
    NT_FENCE();
    z[13] = z[13] - J[72] * z[12] - J[73] * z[2] - J[74] * z[48] - J[75] * z[45] - J[76] * z[52];
    NT_FENCE();
    z[25] = z[25] - J[65] * z[18] - J[66] * z[12] - J[67] * z[2] - J[68] * z[48] - J[69] * z[45] - J[70] * z[53] - J[71] * z[47];
    NT_FENCE();
    z[51] = z[51] - J[64] * z[49];
    NT_FENCE();
    z[0] = z[0] - J[63] * z[42];
    NT_FENCE();
    z[5] = z[5] - J[58] * z[20] - J[59] * z[12] - J[60] * z[2] - J[61] * z[48] - J[62] * z[46];
    NT_FENCE();
    z[54] = z[54] - J[55] * z[20] - J[56] * z[48] - J[57] * z[46];
    NT_FENCE();
    z[35] = z[35] - J[54] * z[43];
    NT_FENCE();
    z[15] = z[15] - J[49] * z[13] - J[50] * z[14] - J[51] * z[12] - J[52] * z[44] - J[53] * z[52];
    NT_FENCE();
    z[19] = z[19] - J[45] * z[2] - J[46] * z[48] - J[47] * z[45] - J[48] * z[53];
    NT_FENCE();
    z[37] = z[37] - J[43] * z[42] - J[44] * z[43];
    NT_FENCE();
    z[39] = z[39] - J[42] * z[42];
    NT_FENCE();
    z[26] = z[26] - J[36] * z[25] - J[37] * z[14] - J[38] * z[18] - J[39] * z[12] - J[40] * z[53] - J[41] * z[52];
    NT_FENCE();
    z[31] = z[31] - J[35] * z[42];
    NT_FENCE();
    z[36] = z[36] - J[33] * z[42] - J[34] * z[43];
    NT_FENCE();
    z[29] = z[29] - J[30] * z[28] - J[31] * z[43] - J[32] * z[47];
    NT_FENCE();
    z[33] = z[33] - J[29] * z[42];
    NT_FENCE();
    z[38] = z[38] - J[28] * z[42];
    NT_FENCE();
    z[17] = z[17] - J[24] * z[5] - J[25] * z[12] - J[26] * z[48] - J[27] * z[44];
    NT_FENCE();
    z[3] = z[3] - J[19] * z[0] - J[20] * z[51] - J[21] * z[42] - J[22] * z[4] - J[23] * z[49];
    NT_FENCE();
    z[32] = z[32] - J[18] * z[42];
    NT_FENCE();
    z[40] = z[40] - J[11] * z[38] - J[12] * z[39] - J[13] * z[37] - J[14] * z[42] - J[15] * z[41] - J[16] * z[18] - J[17] * z[43];
    NT_FENCE();
    z[6] = z[6] - J[0] * z[32] - J[1] * z[38] - J[2] * z[33] - J[3] * z[36] - J[4] * z[31] - J[5] * z[35] - J[6] * z[34] - J[7] * z[30] - J[8] * z[42] - J[9] * z[12] - J[10] * z[43];
}
}  // namespace rpb
