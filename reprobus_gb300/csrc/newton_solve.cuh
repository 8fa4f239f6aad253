// newton_solve.cuh — Newton iteration on the generated step equations
// (newton_gen.cuh), shared by the CUDA kernels and host-side checks.
//
// x = (ck(1..42), cc(1..15)). An iteration evaluates the residual R(x) in
// FP64 (nt_residual_*), then nt_linear_step: the Jacobian in TJ (double for
// the plain solver, float for the mixed one), scaled to relative units with
// s_i = max(|x_i|, 1e-20 hnm) (the accuracy criterion concerns species above
// 1e-20 mol/mol): J'_ij = J_ij s_j / s_i and b_i = -R_i / s_i, all in TJ; the
// sparse LU on the generated fill pattern; the scaled step y; and the FP64
// update x_i += s_i y_i. A component that the step would make negative is set
// to a tenth of its value (the fixed point is non-negative). The iteration has
// converged when max_i |y_i| < tol.
#pragma once
#include "newton_gen.cuh"

namespace rpb {

// read-only strided view: v[i] = p[i * s] (structure-of-arrays over cells)
template <typename T>
struct SP {
    const T* p;
    int s;
    __device__ __forceinline__ T operator[](int i) const { return p[(size_t)i * s]; }
};
// writable strided view
template <typename T>
struct SPW {
    T* p;
    int s;
    __device__ __forceinline__ T& operator[](int i) const { return p[(size_t)i * s]; }
};

// one linearised step from the residual R at x; x updated in FP64.
// KT/tjT/hetT: rate views in TJ; J: NT_NSLOT slots of TJ storage.
// Returns false when the step is not finite; *step = max |y_i|.
template <typename TJ, typename FF, typename PK, typename PXD, typename PRD, typename PJ>
__device__ __forceinline__ bool nt_linear_step(const FF& FT, PK KT, PK tjT, PK hetT, bool day, double hnm, PXD x,
                                               PRD R, PJ J, TJ* step) {
    TJ s[NT_NX], rs[NT_NX], xt[NT_NX], b[NT_NX];
    const double floor_ = 1e-20 * hnm;
#pragma unroll
    for (int i = 0; i < NT_NX; i++) {
        const double xi = x[i];
        s[i] = (TJ)fmax(fabs(xi), floor_);
        rs[i] = TJ(1) / s[i];
        xt[i] = (TJ)xi;
    }
    if (day)
        nt_jacobian_day<TJ>(FT, KT, tjT, hetT, (const TJ*)xt, J);
    else
        nt_jacobian_night<TJ>(FT, KT, tjT, hetT, (const TJ*)xt, J);
    nt_scale<TJ>(J, s, rs);
    nt_lu<TJ>(J, (TJ)1e-30);
#pragma unroll
    for (int i = 0; i < NT_NX; i++) b[i] = (TJ)(-R[i]) * rs[i];
    nt_solve<TJ>(J, b);
    TJ st = 0;
    bool finite = true;
#pragma unroll
    for (int i = 0; i < NT_NX; i++) {
        const double xo = x[i];
        double xn = xo + (double)(b[i] * s[i]);
        if (xo > 0. && xn < 0.) xn = 0.1 * xo;
        const TJ y = fabs(b[i]);
        if (!(y <= TJ(1e30))) finite = false;
        st = fmax(st, y);
        x[i] = xn;
    }
    *step = st;
    return finite;
}

struct NtIn {
    NtFix F;
    const double* K;    // 99 rate constants
    const double* tj;   // 41 photolysis rates
    const double* het;  // 9 heterogeneous rates
    const double* ck0;  // 42 start-of-step number densities
    bool day;
};

// whole iteration on one cell with local storage (host checks); returns
// iterations used (>= 1) when converged, -1 otherwise; x updated in place
template <typename TJ>
__device__ __forceinline__ int nt_newton(const NtIn& in, const TJ* KT, const TJ* tjT, const TJ* hetT,
                                         const NtFixT<TJ>& FT, double* x, int maxit, double tol,
                                         double* last_step) {
    double R[NT_NX];
    TJ J[NT_NSLOT];
    *last_step = 1e300;
    for (int it = 1; it <= maxit; it++) {
        if (in.day)
            nt_residual_day<double>(in.F, in.K, in.tj, in.het, in.ck0, (const double*)x, R);
        else
            nt_residual_night<double>(in.F, in.K, in.tj, in.het, in.ck0, (const double*)x, R);
        TJ st;
        const bool ok = nt_linear_step<TJ>(FT, KT, tjT, hetT, in.day, in.F.hnm, x, (const double*)R, J, &st);
        *last_step = (double)st;
        if (!ok) return -1;
        if (st < (TJ)tol) return it;
    }
    return -1;
}

}  // namespace rpb
