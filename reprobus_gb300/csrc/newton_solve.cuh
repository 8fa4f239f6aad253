// newton_solve.cuh — per-cell Newton iteration on the generated step equations
// (newton_gen.cuh), shared by the CUDA kernels and host-side checks.
//
// x = (ck(1..42), cc(1..15)). Each iteration evaluates the residual R(x) in
// FP64 and the Jacobian in TJ (double for the plain solver, float for the
// mixed one), scales the system to relative units with s_i = max(|x_i|,
// 1e-20 hnm) (the accuracy criterion concerns species above 1e-20 mol/mol):
// J'_ij = J_ij s_j / s_i, b_i = -R_i / s_i, all in TJ; factorises J' (sparse
// LU on the generated fill pattern), solves for the scaled step y and updates
// x_i += s_i y_i in FP64. A component that the step would drive below a tenth
// of its value is clipped there (the fixed point is non-negative). Converged
// when max_i |y_i| < tol.
#pragma once
#include "newton_gen.cuh"

namespace rpb {

struct NtIn {
    NtFix F;
    const double* K;    // 99 rate constants
    const double* tj;   // 41 photolysis rates
    const double* het;  // 9 heterogeneous rates
    const double* ck0;  // 42 start-of-step number densities
    bool day;
};

// returns iterations used (>= 1) when converged, -1 otherwise; x updated in place
template <typename TJ>
__device__ __forceinline__ int nt_newton(const NtIn& in, const TJ* KT, const TJ* tjT, const TJ* hetT,
                                         const NtFixT<TJ>& FT, double* x, int maxit, double tol,
                                         double* last_step) {
    double R[NT_NX];
    TJ s[NT_NX], rs[NT_NX], xt[NT_NX];
    TJ J[NT_NSLOT];
    TJ b[NT_NX];
    const double floor_ = 1e-20 * in.F.hnm;
    *last_step = 1e300;
#pragma unroll 1
    for (int it = 1; it <= maxit; it++) {
        if (in.day)
            nt_residual_day<double>(in.F, in.K, in.tj, in.het, in.ck0, x, R);
        else
            nt_residual_night<double>(in.F, in.K, in.tj, in.het, in.ck0, x, R);
#pragma unroll
        for (int i = 0; i < NT_NX; i++) {
            s[i] = (TJ)fmax(fabs(x[i]), floor_);
            rs[i] = TJ(1) / s[i];
            xt[i] = (TJ)x[i];
        }
        if (in.day)
            nt_jacobian_day<TJ>(FT, KT, tjT, hetT, xt, J);
        else
            nt_jacobian_night<TJ>(FT, KT, tjT, hetT, xt, J);
        nt_scale<TJ>(J, s, rs);
        nt_lu<TJ>(J, (TJ)1e-30);
#pragma unroll
        for (int i = 0; i < NT_NX; i++) b[i] = (TJ)(-R[i]) * rs[i];
        nt_solve<TJ>(J, b);
        TJ step = 0;
        bool finite = true;
#pragma unroll
        for (int i = 0; i < NT_NX; i++) {
            const double xo = x[i];
            double xn = xo + (double)(b[i] * s[i]);
            if (xo > 0. && xn < 0.) xn = 0.1 * xo;
            const TJ y = fabs(b[i]);
            if (!(y <= TJ(1e30))) finite = false;
            step = fmax(step, y);
            x[i] = xn;
        }
        *last_step = (double)step;
        if (!finite) return -1;
        if (step < (TJ)tol) return it;
    }
    return -1;
}

}  // namespace rpb
