// newton_solve.cuh — one Newton iteration on the generated step equations
// (newton_gen.cuh), shared by the CUDA kernels and host-side checks.
//
// x = (ck(1..42), cc(1..15)). An iteration evaluates the scaled Jacobian in TJ
// (double for the plain solver, float for the mixed one) into the cell's
// matrix slots, the residual R(x) in FP64, the right-hand side z_i = -R_i / s_i
// in TJ, the sparse Crout factorisation with fused forward substitution and the
// back substitution in TJ, and the FP64 update x_i += s_i z_i. The scales
// s_i = 2^floor(log2(max(|x_i|, 1e-20 hnm))) are powers of two (the accuracy
// criterion concerns species above 1e-20 mol/mol), so scaling rounds nothing.
// A component that the step would make negative is set to a tenth of its
// value (the fixed point is non-negative). The iteration has converged when
// max_i |z_i| < tol.
#pragma once
#include <cstdint>
#include "newton_gen.cuh"
#ifndef __CUDACC__
#define __noinline__
#endif

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
// the NT_NSLOT matrix slots of one cell with a compile-time stride
// (shared memory, slot-major: slot q of lane t at base[q * STRIDE + t])
template <typename T, int STRIDE>
struct SJ {
    static constexpr int stride = STRIDE;
    T* p;
    __device__ __forceinline__ T& operator[](int q) const { return p[q * STRIDE]; }
};

// write-only view of the same slots for the Jacobian: each store is an
// explicit shared-memory store, so the compiler knows that storing the
// Jacobian never changes global memory and may keep the record values and
// the iterate it has read in registers across the stores
#ifdef __CUDACC__
template <typename T, int STRIDE>
struct SJW {
    uint32_t a;  // shared-window address of slot 0 of this lane
    struct Ref {
        uint32_t q;
        __device__ __forceinline__ void operator=(float v) const {
            asm volatile("st.shared.f32 [%0], %1;" ::"r"(q), "f"(v));
        }
        __device__ __forceinline__ void operator=(double v) const {
            asm volatile("st.shared.f64 [%0], %1;" ::"r"(q), "d"(v));
        }
    };
    __device__ __forceinline__ Ref operator[](int s) const { return Ref{a + (uint32_t)(s * STRIDE * sizeof(T))}; }
};
template <typename T, int STRIDE>
__device__ __forceinline__ SJW<T, STRIDE> nt_store_view(SJ<T, STRIDE> J) {
    return SJW<T, STRIDE>{(uint32_t)__cvta_generic_to_shared(J.p)};
}
#endif

constexpr double NT_TINY = 1e-30;   // pivot guard of the factorisation

// right-hand side z_i = -R_i / s_i of the day or night equations into z (a
// register array or shared-memory slots): each R_i (FP64) is scaled and
// rounded to TJ as soon as the residual produces it
template <typename TJ, typename PZ>
struct NtRhsRef {
    PZ z;
    int i;
    double xi;
    int fh;
    __device__ __forceinline__ void operator=(double r) const {
        z[i] = nt_cvt<TJ>(-r) * nt_rscale<TJ>(nt_exp_hi(xi), fh);
    }
};
template <typename TJ, typename PZ>
struct NtRhsOut {
    PZ z;
    const double* x;
    int fh;
    __device__ __forceinline__ NtRhsRef<TJ, PZ> operator[](int i) const { return NtRhsRef<TJ, PZ>{z, i, x[i], fh}; }
};
template <typename TJ, typename FF, typename PK, typename PC, typename PZ>
__device__ __forceinline__ void nt_rhs(bool day, const FF& F, PK K, PK tj, PK het, PC ck0,
                                       const double* __restrict__ x, double floor_, PZ z) {
    const NtRhsOut<TJ, PZ> R{z, x, nt_exp_hi(floor_)};
    if (day)
        nt_residual_day<double>(F, K, tj, het, ck0, x, R);
    else
        nt_residual_night<double>(F, K, tj, het, ck0, x, R);
}
// the same as a call of its own (z in shared memory)
template <typename TJ, typename FF, typename PK, typename PC, typename PZ>
__device__ __noinline__ void nt_rhs_fn(bool day, const FF& F, PK K, PK tj, PK het, PC ck0,
                                       const double* __restrict__ x, double floor_, PZ z) {
    nt_rhs<TJ>(day, F, K, tj, het, ck0, x, floor_, z);
}

// z slots after the matrix slots of a shared-memory cell view
template <typename T, int STRIDE>
struct SJZ {
    T* p;
    __device__ __forceinline__ T& operator[](int i) const { return p[(NT_NSLOT + i) * STRIDE]; }
};

template <typename PJ>
struct nt_is_sj {
    static constexpr bool value = false;
};
template <typename T, int STRIDE>
struct nt_is_sj<SJ<T, STRIDE>> {
    static constexpr bool value = true;
};

// the Jacobian of the day or night equations as a call of its own, so that
// its register allocation does not meet the residual's and the solve's
template <typename TJ, typename FFT, typename PKT, typename PJ>
__device__ __noinline__ void nt_jacobian_fn(bool day, const FFT& FT, PKT KT, PKT tjT, PKT hetT, const double* x,
                                             double floor_, PJ J) {
    if (day)
        nt_jacobian_day<TJ>(FT, KT, tjT, hetT, x, floor_, J);
    else
        nt_jacobian_night<TJ>(FT, KT, tjT, hetT, x, floor_, J);
}
template <typename TJ, typename FFT, typename PKT, typename PJ>
__device__ __forceinline__ void nt_jacobian_call(bool day, const FFT& FT, PKT KT, PKT tjT, PKT hetT, const double* x,
                                                 double floor_, PJ J) {
#ifdef __CUDA_ARCH__
    if constexpr (nt_is_sj<PJ>::value && sizeof(TJ) == 4)  // (FP64: the freedom costs spills)
        nt_jacobian_fn<TJ>(day, FT, KT, tjT, hetT, x, floor_, nt_store_view(J));
    else
        nt_jacobian_fn<TJ>(day, FT, KT, tjT, hetT, x, floor_, J);
#else
    if (day)
        nt_jacobian_day<TJ>(FT, KT, tjT, hetT, x, floor_, J);
    else
        nt_jacobian_night<TJ>(FT, KT, tjT, hetT, x, floor_, J);
#endif
}

// One iteration from x (updated in place, FP64). F/K/tj/het/ck0: FP64 inputs
// of the residual; FT/KT/tjT/hetT: the same in TJ for the Jacobian. J: the
// cell's NT_NSLOT matrix slots. Returns false when the step is not finite;
// *step = max |z_i|.
template <typename TJ, typename PZ>
__device__ __forceinline__ bool nt_update(double* x, double floor_, PZ z, TJ* step, bool active);

// ZSHARED (device only): z in NT_NX shared-memory slots after the matrix (the
// residual as a call of its own) instead of registers (residual inlined).
template <typename TJ, bool ZSHARED = false, typename FF, typename PK, typename PC, typename FFT, typename PKT,
          typename PJ>
__device__ __forceinline__ bool nt_iterate(const FF& F, PK K, PK tj, PK het, PC ck0, const FFT& FT, PKT KT, PKT tjT,
                                           PKT hetT, bool day, double* x, PJ J, TJ* step, bool active = true) {
    const double floor_ = 1e-20 * F.hnm;
    nt_jacobian_call<TJ>(day, FT, KT, tjT, hetT, x, floor_, J);
    NT_FENCE();
#ifdef __CUDA_ARCH__
    if constexpr (ZSHARED) {
        const SJZ<TJ, PJ::stride> z{J.p};
        // the residual stores z through explicit shared-memory stores (as the
        // Jacobian does its slots), so the record values it reads stay in registers
        const SJW<TJ, PJ::stride> zw{(uint32_t)__cvta_generic_to_shared(J.p) +
                                     (uint32_t)(NT_NSLOT * PJ::stride * sizeof(TJ))};
        nt_rhs_fn<TJ>(day, F, K, tj, het, ck0, x, floor_, zw);
        nt_factor_solve<TJ>(J, z, TJ(NT_TINY));
        return nt_update<TJ>(x, floor_, z, step, active);
    }
#endif
    TJ z[NT_NX];
    nt_rhs<TJ>(day, F, K, tj, het, ck0, x, floor_, (TJ*)z);
    nt_factor_solve<TJ>(J, (TJ*)z, TJ(NT_TINY));
    return nt_update<TJ>(x, floor_, (const TJ*)z, step, active);
}

// FP64 update x_i += s_i z_i (negative results clipped to x_i / 10);
// returns false when a step is not finite; *step = max |z_i|. active false:
// a lane that runs the iteration only to keep its warp converged writes nothing.
template <typename TJ, typename PZ>
__device__ __forceinline__ bool nt_update(double* x, double floor_, PZ z, TJ* step, bool active) {
    const int fh = nt_exp_hi(floor_);
    TJ st = 0;
    bool finite = true;
#pragma unroll
    for (int i = 0; i < NT_NX; i++) {
        const TJ zi = z[i];
        const double xo = x[i];
        double xn = xo + nt_widen(zi) * nt_scale<double>(nt_exp_hi(xo), fh);
        if (xo > 0. && xn < 0.) xn = 0.1 * xo;
        const TJ y = fabs(zi);
        if (!(y <= TJ(1e30))) finite = false;
        st = fmax(st, y);
        if (active) x[i] = xn;
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
inline int nt_newton(const NtIn& in, const TJ* KT, const TJ* tjT, const TJ* hetT, const NtFixT<TJ>& FT, double* x,
                     int maxit, double tol, double* last_step) {
    TJ J[NT_NSLOT];
    *last_step = 1e300;
    for (int it = 1; it <= maxit; it++) {
        TJ st;
        const bool ok = nt_iterate<TJ>(in.F, in.K, in.tj, in.het, in.ck0, FT, KT, tjT, hetT, in.day, x, J, &st);
        *last_step = (double)st;
        if (!ok) return -1;
        if (st < (TJ)tol) return it;
    }
    return -1;
}

}  // namespace rpb
