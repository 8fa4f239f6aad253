// Host build of the generated step equations and of the Newton iteration
// (reprobus_gb300/csrc/newton_gen.cuh, newton_solve.cuh) for CPU checks of
// the generator: residual, Jacobian against finite differences, and Newton
// against the oracle's fixed point. Compiled by tests/test_newton_equations.py.
#include <cmath>
#include <cstring>
#include <cstdlib>
using std::fabs;
using std::fmax;
using std::fmin;
using std::sqrt;
#include "../reprobus_gb300/csrc/chem_enums.h"
#include "../reprobus_gb300/csrc/newton_solve.cuh"

using namespace rpb;

static NtFix fix_from(const double* f) {
    NtFix F;
    F.o2 = f[0]; F.n2 = f[1]; F.h2 = f[2]; F.co2 = f[3]; F.hnm = f[4]; F.parthno3 = f[5]; F.parth2o = f[6];
    F.parthcl = f[7]; F.parthbr = f[8]; F.rain_hno3 = f[9]; F.rain_hcl = f[10]; F.rain_hbr = f[11];
    F.rain_h2o2 = f[12]; F.dt = f[13];
    return F;
}

template <typename T>
static NtFixT<T> fix_t(const NtFix& F) {
    NtFixT<T> G;
    G.o2 = (T)F.o2; G.n2 = (T)F.n2; G.h2 = (T)F.h2; G.co2 = (T)F.co2; G.hnm = (T)F.hnm;
    G.parthno3 = (T)F.parthno3; G.parth2o = (T)F.parth2o; G.parthcl = (T)F.parthcl; G.parthbr = (T)F.parthbr;
    G.rain_hno3 = (T)F.rain_hno3; G.rain_hcl = (T)F.rain_hcl; G.rain_hbr = (T)F.rain_hbr;
    G.rain_h2o2 = (T)F.rain_h2o2; G.dt = (T)F.dt;
    return G;
}

extern "C" {
int nt_host_nx(void) { return NT_NX; }
int nt_host_nslot(void) { return NT_NSLOT; }

void nt_host_residual(const double* K, const double* tj, const double* het, const double* fix, const double* ck0,
                      int day, const double* x, double* R) {
    NtFix F = fix_from(fix);
    if (day)
        nt_residual_day<double>(F, K, tj, het, ck0, x, R);
    else
        nt_residual_night<double>(F, K, tj, het, ck0, x, R);
}

// dense scaled Jacobian J'_ij = dR_i/dx_j s_j / s_i (row-major NX x NX,
// original numbering, power-of-two scales of nt_pow2_scale), FP64
void nt_host_jacobian(const double* K, const double* tj, const double* het, const double* fix, int day,
                      const double* x, double* Jd) {
    NtFix F = fix_from(fix);
    double J[NT_NSLOT];
    const double floor_ = 1e-20 * F.hnm;
    if (day)
        nt_jacobian_day<double>(F, K, tj, het, x, floor_, J);
    else
        nt_jacobian_night<double>(F, K, tj, het, x, floor_, J);
    memset(Jd, 0, sizeof(double) * NT_NX * NT_NX);
    for (int q = 0; q < NT_NA; q++) Jd[NT_A_I[q] * NT_NX + NT_A_J[q]] = J[q];
    for (int q = 0; q < NT_NCONST; q++) Jd[NT_CONST_I[q] * (NT_NX + 1)] = NT_CONST_V[q];
}

// the residual and the scaled Jacobian assembled from the W row groups of the
// warps-per-cell kernel (each row written by exactly one group; rows a group
// does not own keep the NaN they start with)
void nt_host_residual_groups(int W, const double* K, const double* tj, const double* het, const double* fix,
                             const double* ck0, int day, const double* x, double* R) {
    NtFix F = fix_from(fix);
    for (int i = 0; i < NT_NX; i++) R[i] = NAN;
    for (int g = 0; g < W; g++) {
        if (W == 2) {
            if (day) nt_residual_day_w2<double>(g, F, K, tj, het, ck0, x, R);
            else nt_residual_night_w2<double>(g, F, K, tj, het, ck0, x, R);
        } else {
            if (day) nt_residual_day_w4<double>(g, F, K, tj, het, ck0, x, R);
            else nt_residual_night_w4<double>(g, F, K, tj, het, ck0, x, R);
        }
    }
}

void nt_host_jacobian_groups(int W, const double* K, const double* tj, const double* het, const double* fix, int day,
                             const double* x, double* Jd) {
    NtFix F = fix_from(fix);
    double J[NT_NSLOT];
    for (int q = 0; q < NT_NSLOT; q++) J[q] = NAN;
    const double floor_ = 1e-20 * F.hnm;
    for (int g = 0; g < W; g++) {
        if (W == 2) {
            if (day) nt_jacobian_day_w2<double>(g, F, K, tj, het, x, floor_, J);
            else nt_jacobian_night_w2<double>(g, F, K, tj, het, x, floor_, J);
        } else {
            if (day) nt_jacobian_day_w4<double>(g, F, K, tj, het, x, floor_, J);
            else nt_jacobian_night_w4<double>(g, F, K, tj, het, x, floor_, J);
        }
    }
    memset(Jd, 0, sizeof(double) * NT_NX * NT_NX);
    for (int q = 0; q < NT_NA; q++) Jd[NT_A_I[q] * NT_NX + NT_A_J[q]] = J[q];
    for (int q = 0; q < NT_NCONST; q++) Jd[NT_CONST_I[q] * (NT_NX + 1)] = NT_CONST_V[q];
}

// Newton from x (in/out); mixed: float Jacobian. Returns iterations or -1.
int nt_host_newton(const double* K, const double* tj, const double* het, const double* fix, const double* ck0,
                   int day, double* x, int maxit, double tol, int mixed, double* last_step) {
    NtIn in;
    in.F = fix_from(fix);
    in.K = K; in.tj = tj; in.het = het; in.ck0 = ck0; in.day = day != 0;
    if (mixed) {
        float Kf[K_COUNT], tf[41], hf[9];
        for (int i = 0; i < K_COUNT; i++) Kf[i] = (float)K[i];
        for (int i = 0; i < 41; i++) tf[i] = (float)tj[i];
        for (int i = 0; i < 9; i++) hf[i] = (float)het[i];
        return nt_newton<float>(in, Kf, tf, hf, fix_t<float>(in.F), x, maxit, tol, last_step);
    }
    return nt_newton<double>(in, K, tj, het, fix_t<double>(in.F), x, maxit, tol, last_step);
}
}
