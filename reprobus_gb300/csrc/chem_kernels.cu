// chem_kernels.cu — GB300 (sm_103a) kernels and C-ABI of the REPROBUS
// chemistry step (include/reprobus_chem.h).
//
// Launch structure of one step (rows ilat0..ilat1, levels 1..nivbas):
//   k_columns  one thread per column: the vertical prefix sums of total
//              (F:5153-5186) and jno (JNO:107-126) and the level-1 zenith
//              angle (JNO:139) -> column scratch (3 doubles per cell + 1 per
//              column)
//   k_chem     one thread per cell: setup, zenith, phot+jno, analytic+hetero,
//              rate constants, rainout, the niter fixed-point passes,
//              write-back and (fused) conserv + clamps  (F:800-2410, 2526-2616)
//   k_tail     (fused, nivbas < niv) clamps and HNO3-gas copy of the levels
//              below the chemistry (F:431-450)
// All arrays keep the reference's Fortran layout, lon fastest, so a warp's
// loads of one species plane are coalesced.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <new>

#include "../../include/reprobus_chem.h"
#include "chem_params.cuh"
#include "newton_gen.cuh"
#include "newton_launch.h"
#include "mlp_net.h"
#include "handle_info.h"

using namespace rpb;

// ----------------------------------------------------------------------------
// error reporting
// ----------------------------------------------------------------------------
static thread_local char g_err[512] = "";

static int set_err(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

// the same error channel for the other translation units (not exported)
extern "C" __attribute__((visibility("hidden"))) int reprobus_set_error(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

#define CUDA_TRY(x)                                                                                          \
    do {                                                                                                     \
        cudaError_t e_ = (x);                                                                                \
        if (e_ != cudaSuccess) return set_err(REPROBUS_ERR_CUDA, "%s: %s (%s:%d)", #x, cudaGetErrorString(e_), \
                                              __FILE__, __LINE__);                                           \
    } while (0)

// Cells are numbered i + nlon (r + nrows k) over the longitudes (i), the
// step's rows (r) and the chemistry levels (k); columns i + nlon r. The
// per-cell kernels of the rate stage, the start and the write-back take the
// cells of a window of rows win_r0 .. win_r0 + win_nr - 1: thread t handles
// the t-th cell (column) of the window, the identity when the window is the
// whole range. The host-array entry point runs those phases row chunk by row
// chunk while the copies of the other chunks are in flight.
__device__ __forceinline__ int win_cell(const Params& P, int t) {
    const int i = t % P.nlon, rest = t / P.nlon;
    return i + P.nlon * (P.win_r0 + rest % P.win_nr + P.nrows * (rest / P.win_nr));
}
__device__ __forceinline__ int win_col(const Params& P, int t) { return t % P.nlon + P.nlon * (P.win_r0 + t / P.nlon); }

// ----------------------------------------------------------------------------
// k_columns — vertical prefix sums, total F:5172-5184 and jno JNO:109-126
// ----------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_columns(Params P) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P.win_ncol) return;
    const int col = win_col(P, t);
    const int i = col % P.nlon;
    const int j = P.ilat0 + col / P.nlon;
    const size_t pl = plane3(P);
    const double zcmt = 2.120e20;                      // total
    const double zcmt2 = 287.0 / (1.38e-23 * 9.81);    // jno
    const double r_o2 = 0.2095;
    double* o3t = P.col;
    double* colo2 = P.col + P.ncell;
    double* colno = P.col + 2 * (size_t)P.ncell;
    double* sza_top = P.col + 3 * (size_t)P.ncell;
    // level 1
    size_t g = (size_t)i + (size_t)P.nlon * j;
    double p_prev = P.trajpre[P.trajoff + g];
    double hnm_prev = p_prev / (P.trajtem[P.trajoff + g] * 1.38e-19);
    double o3_prev = P.hc[g + pl * 4];
    double no_prev = P.hc[g + pl * 7] * hnm_prev;  // cc(:,:,8) = hc*hnm
    double a_o3 = o3_prev * hnm_prev * 6.8e5;
    double a_o2 = 6.8e+05 * r_o2 * hnm_prev;
    double a_no = 6.8e+05 * no_prev;
    o3t[col] = a_o3;
    colo2[col] = a_o2;
    colno[col] = a_no;
    sza_top[col] = cell_zenith(P.sc, P.trajlon[P.trajoff + g], P.trajlat[P.trajoff + g]);
    for (int k = 1; k < P.nivbas; k++) {
        g += (size_t)P.nlon * P.nlat;
        double p = P.trajpre[P.trajoff + g];
        double hnm = p / (P.trajtem[P.trajoff + g] * 1.38e-19);
        double o3 = P.hc[g + pl * 4];
        double no = P.hc[g + pl * 7] * hnm;
        double dp = (p - p_prev) * 100.;
        dp = fmax(dp, 0.);
        a_o3 = a_o3 + zcmt * (o3 + o3_prev) * .5 * dp;
        a_o2 = a_o2 + zcmt2 * (r_o2 + r_o2) * 0.5 * dp * 1.e-4;
        a_no = a_no + zcmt2 * (no_prev / hnm_prev + no / hnm) * 0.5 * dp * 1.e-4;
        const size_t c = (size_t)col + (size_t)P.ncol * k;
        o3t[c] = a_o3;
        colo2[c] = a_o2;
        colno[c] = a_no;
        p_prev = p;
        hnm_prev = hnm;
        o3_prev = o3;
        no_prev = no;
    }
}

// ----------------------------------------------------------------------------
// rate stage of one cell (F:800-1338): everything chem3d computes before its
// iteration. Shared by the fixed-pass kernel and the Newton kernels.
// ----------------------------------------------------------------------------
struct CellPro {
    CellFix F;
    double ck0[NBCON];
    double cc0[NCM];
    double tj[NPHOT];
    double K[NRATE];
    Aerosol A;
    double o3t;
    size_t g;
    int k;
};

// LS: the block's threads pass each phase (loads, zenith, photolysis,
// aerosol, rates) between the same barriers, so that the warps of an SM
// fetch the same code at the same time; every thread of the block must call
// it (store = false: a thread without a cell of its own, which recomputes a
// valid cell and writes nothing).
template <bool DIAG, bool LS = false>
__device__ __forceinline__ void cell_prologue(const Params& P, int cell, CellPro& C, bool store = true) {
    const int i = cell % P.nlon;
    const int rest = cell / P.nlon;
    const int col = cell % P.ncol;
    const int k = rest / P.nrows;
    const int j = P.ilat0 + rest % P.nrows;
    const size_t g = (size_t)i + (size_t)P.nlon * ((size_t)j + (size_t)P.nlat * k);
    const size_t pl = plane3(P);
    C.g = g;
    C.k = k;
    CellFix& F = C.F;
    // setup F:800-833
    const double t = P.trajtem[P.trajoff + g];
    const double pm = P.trajpre[P.trajoff + g];
    F.hnm = div64(P.trajpre[P.trajoff + g], P.trajtem[P.trajoff + g] * 1.38e-19);
    F.n2 = 0.78 * F.hnm;
    F.o2 = 0.21 * F.hnm;
    F.co2 = 360.e-6 * F.hnm;
    F.h2 = 5.e-7 * F.hnm;
#pragma unroll
    for (int n = 0; n < NBCON; n++) C.ck0[n] = P.qj1[g + pl * n] * F.hnm;
#pragma unroll
    for (int n = 0; n < NCM; n++) C.cc0[n] = P.hc[g + pl * n] * F.hnm;
    if (LS) __syncthreads();
    // zenith F:845-851
    F.sza = cell_zenith(P.sc, P.trajlon[P.trajoff + g], P.trajlat[P.trajoff + g]);
    if (!DIAG && store) P.sza3d[g] = F.sza;
    if (LS) __syncthreads();
    // phot + jno F:857, F:5043-5146
#pragma unroll
    for (int n = 0; n < NPHOT; n++) C.tj[n] = 0.;
    C.o3t = P.col[cell];
    if (F.sza <= 95.) cell_phot(P.ajl, P.o3up, P.alt[g], F.sza, C.o3t, C.tj);
    const double sza_top = P.col[3 * (size_t)P.ncell + col];
    if (sza_top <= 89.0)
        C.tj[J_no] = cell_jno(sza_top, F.hnm, P.col[(size_t)P.ncell + cell], P.col[2 * (size_t)P.ncell + cell], C.o3t);
    if (LS) __syncthreads();
    // heterogeneous init + analytic F:864-912
    Aerosol& A = C.A;
#pragma unroll
    for (int m = 0; m < 9; m++) A.het[m] = 0.;
    A.parthno3 = 1.;
    A.parthno3sl = 1.;
    A.parth2o = 1.;
    A.parthcl = 1.;
    A.vsed = 0.;
    A.surf = 0.;
    if (k >= P.nivhau - 1) {
        cell_aerosol(t, pm, F.hnm, C.ck0, A);
        if (!DIAG && store) P.surfarea[g] = A.surf;
    }
    F.parthno3 = A.parthno3;
    F.parth2o = A.parth2o;
    F.parthcl = A.parthcl;
    F.parthbr = 1.;
    if (!DIAG && store) {
        P.vsed3d[g] = A.vsed;
        P.parth2osed[g] = A.parth2o;
        P.parthno3sed[g] = A.parthno3sl;
    }
    if (LS) __syncthreads();
    // rate constants F:920-1306
    cell_rates(P.sc.troe, P.sc.ltroe, t, F.hnm, pm, C.K);
    // rainout F:1315-1338
    const double rain_rate = 1.e-6;
    const bool rain = div64(C.ck0[2], F.hnm) >= 100.e-6;
    F.rain_hno3 = rain ? rain_rate : 0.;
    F.rain_hno4 = 0.;
    F.rain_hcl = rain ? rain_rate : 0.;
    F.rain_hbr = rain ? rain_rate : 0.;
    F.rain_h2o2 = rain ? rain_rate : 0.;
    F.rain_ch2o = 0.;
    F.rain_ch3o2h = 0.;
}

// fmax(v, 1e-30) on the integer pipe: below 1e-30 (negative, zero or
// smaller), the signed integer of a double's bits is below that of 1e-30;
// NaN gives 1e-30, as fmax does
__device__ __forceinline__ double clamp_1e30(double v) {
    long long b;
    memcpy(&b, &v, 8);
    const long long lo = 0x39b4484bfeebc2a0LL;  // the bits of 1e-30
    const bool nan = (b & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
    return (b < lo || nan) ? 1.e-30 : v;
}

// write-back F:2380-2410, then (fused) conserv F:2539-2613 and clamps F:431-440
// RECIP: number density -> mixing ratio by one reciprocal of hnm and
// products (within an ulp of the reference's divisions, F:2380-2410), for the
// Newton solvers, whose answer is accurate to their tolerance; the reference
// scheme keeps the divisions.
template <bool RECIP = false>
__device__ __forceinline__ void cell_epilogue(const Params& P, const CellPro& C, const double* ck, const double* cc) {
    const size_t pl = plane3(P);
    double q[NBCON], h[NCM];
    if (RECIP) {
        const double rh = div64(1., C.F.hnm);
#pragma unroll
        for (int n = 0; n < NBCON - 1; n++) q[n] = ck[n] * rh;
        q[NBCON - 1] = ck[4] * C.F.parthno3 * rh;
#pragma unroll
        for (int n = 0; n < NCM; n++) h[n] = cc[n] * rh;
    } else {
#pragma unroll
        for (int n = 0; n < NBCON - 1; n++) q[n] = ck[n] / C.F.hnm;
        q[NBCON - 1] = ck[4] * C.F.parthno3 / C.F.hnm;
#pragma unroll
        for (int n = 0; n < NCM; n++) h[n] = cc[n] / C.F.hnm;
    }
    if (P.fuse) cell_conserv(q, h);
    if (P.check) {
        unsigned int bad = 0;
#pragma unroll
        for (int n = 0; n < NBCON; n++) bad += !isfinite(q[n]);
#pragma unroll
        for (int n = 0; n < NCM; n++) bad += !isfinite(h[n]);
        if (bad) atomicAdd(P.nonfinite, (unsigned long long)bad);
    }
    if (P.fuse) {
#pragma unroll
        for (int n = 0; n < NBCON - 1; n++) q[n] = clamp_1e30(q[n]);
    }
#pragma unroll
    for (int n = 0; n < NBCON; n++) P.qj1[C.g + pl * n] = q[n];
#pragma unroll
    for (int n = 0; n < NCM; n++) P.hc[C.g + pl * n] = h[n];
}

// ----------------------------------------------------------------------------
// k_chem — one cell per thread. DIAG: rate stage only, diagnostics out.
// ----------------------------------------------------------------------------
// LS (with NTB threads per block): the rate stage in lock-step, as
// k_nt_setup (threads past the last cell recompute it and write nothing)
template <bool DIAG, int NTB = 128, bool LS = false>
__global__ void __launch_bounds__(NTB, 1) k_chem(Params P) {
    int cell = blockIdx.x * blockDim.x + threadIdx.x;
    const bool own = cell < P.ncell;
    if (!LS && !own) return;
    if (!own) cell = P.ncell - 1;
    CellPro C;
    cell_prologue<DIAG, LS>(P, cell, C, own);
    if (!own) return;
    const CellFix& F = C.F;
    const Aerosol& A = C.A;
    if (DIAG) {
        const size_t nc = (size_t)P.ncell;
        double* d = P.diag + cell;
        d[REPROBUS_DIAG_HNM * nc] = F.hnm;
        d[REPROBUS_DIAG_SZA * nc] = F.sza;
        d[REPROBUS_DIAG_O3T * nc] = C.o3t;
#pragma unroll
        for (int n = 0; n < NPHOT; n++) d[(REPROBUS_DIAG_TJ + n) * nc] = C.tj[n];
#pragma unroll
        for (int m = 0; m < 9; m++) d[(REPROBUS_DIAG_HET + m) * nc] = A.het[m];
        d[REPROBUS_DIAG_PARTHNO3 * nc] = A.parthno3;
        d[REPROBUS_DIAG_PARTHNO3SL * nc] = A.parthno3sl;
        d[REPROBUS_DIAG_PARTH2O * nc] = A.parth2o;
        d[REPROBUS_DIAG_PARTHCL * nc] = A.parthcl;
        d[REPROBUS_DIAG_VSED * nc] = A.vsed;
        d[REPROBUS_DIAG_SURFAREA * nc] = A.surf;
#pragma unroll
        for (int n = 0; n < NRATE; n++) d[(REPROBUS_DIAG_RATE + n) * nc] = C.K[n];
        return;
    }
    double ck[NBCON], cc[NCM];
#pragma unroll
    for (int n = 0; n < NBCON; n++) ck[n] = C.ck0[n];
#pragma unroll
    for (int n = 0; n < NCM; n++) cc[n] = C.cc0[n];
    // fixed-point passes F:1348-2378
#pragma unroll 1
    for (int it = 0; it < P.niter; it++) cell_pass(F, C.K, C.tj, A.het, C.ck0, P.sc.dt, ck, cc);
    cell_epilogue(P, C, ck, cc);
}

// ----------------------------------------------------------------------------
// Newton pipeline: the fixed point of the reference's pass map by Newton's
// method on the generated equations (newton_solve.cuh), Jacobian and LU in TJ
// (double: plain FP64 solver; float: mixed precision), residual and update in
// FP64. One step:
//   k_nt_setup   one thread per cell: rate stage -> the cell's record (rates,
//                fixed constants, zenith angle, ck0, aerosol area; FP32
//                copies for the mixed solver)
//   k_nt_start   one thread per cell: P.npass_plain reference passes from the
//                record's start state -> iterate x; the cell enters the work
//                queue (day cells from the front, night cells from the back).
//                Two kernels rather than one: the rate stage alone is a
//                smaller program for the instruction cache. The mixed solver
//                runs the passes in FP32 (k_nt_start32).
//   k_nt_solve   persistent kernel, one lane per cell, lanes refilled from the
//                queue (newton_kernel.cuh)
//   learned restart (with a network): the cells that missed get the plain
//                start again with the network's features (k_nt_start<3>),
//                the network's prediction (k_mlp_infer), a start from it
//                (k_nt_warm) and a second solve over a queue of their own
//   k_nt_finish  one thread per converged cell: write-back, conserv, clamps
//   k_nt_fallback one thread per cell the solver did not converge after
//                P.maxit iterations: the reference's P.niter passes, then the
//                same write-back
// ----------------------------------------------------------------------------
// the 64 raw features of the warm-start network for one cell: log10 of the 42
// transported and 15 short-lived mixing ratios of the plain start (ck, cc:
// number densities after the plain start's reference passes; floored at
// 1e-30), T, ln p, cos(sza), log10 of the aerosol surface area (floored at
// 1e-12), latitude, time of day (fraction), 0
__device__ __forceinline__ void cell_features(const Params& P, size_t g, double hnm, double sza, double surf,
                                              const double* ck, const double* cc, float* f) {
    // log10 in FP32 (the features are FP32): ratio in FP64, then float
    const double rh = 1. / hnm;
#pragma unroll 6
    for (int n = 0; n < NBCON - 1; n++) f[n] = log10f((float)fmax(ck[n] * rh, 1e-30));
#pragma unroll 5
    for (int n = 0; n < NCM; n++) f[NBCON - 1 + n] = log10f((float)fmax(cc[n] * rh, 1e-30));
    const size_t gi = P.trajoff + g;
    f[57] = (float)P.trajtem[gi];
    f[58] = logf((float)P.trajpre[gi]);
    f[59] = cosf((float)(sza * (PI / 180.)));
    f[60] = log10f((float)fmax(surf, 1e-12));
    f[61] = (float)P.trajlat[gi];
    f[62] = (float)(P.sc.ut / 24.);
    f[63] = 0.f;
}

// 1024 threads per SM (64 registers, the cell's arrays on the stack): the
// rate stage is FP64-pipe bound, and the extra warps keep that pipe fed where
// two 256-thread blocks at 128 registers left it idle a quarter of the time.
template <bool MIXED, int NTB = 128, bool LS = false>
__global__ void __launch_bounds__(NTB, 1024 / NTB) k_nt_setup(Params P) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool own = t < P.win_ncell;
    if (!LS && !own) return;
    const int cell = win_cell(P, own ? t : P.win_ncell - 1);  // lock-step: recompute a valid cell, write nothing
    CellPro C;
    cell_prologue<false, LS>(P, cell, C, own);
    if (!own) return;
    const CellFix& F = C.F;
    const double fx[14] = {F.o2, F.n2, F.h2, F.co2, F.hnm, F.parthno3, F.parth2o, F.parthcl, F.parthbr,
                           F.rain_hno3, F.rain_hcl, F.rain_hbr, F.rain_h2o2, P.sc.dt};
    double* r = P.nt_rec + (size_t)cell * NT_REC;
    // MIXED: the FP32 copies beside the FP64 fields, each value read once
    // from the cell's arrays; by integer operations (nt_cvt: truncated, below
    // 2^-126 zero), not conversion instructions, which issue on the FP64 pipe
    float* q = MIXED ? P.nt_rec32 + (size_t)cell * NT_REC32 : nullptr;
#pragma unroll 4
    for (int n = 0; n < NRATE; n++) {
        const double v = C.K[n];
        r[NT_RK + n] = v;
        if (MIXED) q[NT_RK + n] = nt_cvt<float>(v);
    }
#pragma unroll 4
    for (int n = 0; n < NPHOT; n++) {
        const double v = C.tj[n];
        r[NT_RJ + n] = v;
        if (MIXED) q[NT_RJ + n] = nt_cvt<float>(v);
    }
#pragma unroll
    for (int n = 0; n < 9; n++) {
        const double v = C.A.het[n];
        r[NT_RH + n] = v;
        if (MIXED) q[NT_RH + n] = nt_cvt<float>(v);
    }
#pragma unroll
    for (int n = 0; n < 14; n++) {
        r[NT_RF + n] = fx[n];
        if (MIXED) q[NT_RF + n] = nt_cvt<float>(fx[n]);
    }
    r[NT_RSZA] = F.sza;
    if (MIXED) q[NT_RSZA] = nt_cvt<float>(F.sza);
    r[NT_RSURF] = C.A.surf;
#pragma unroll 4
    for (int n = 0; n < NBCON; n++) r[NT_RCK0 + n] = C.ck0[n];
}

// a cell into the work queue: day cells from the front of the list, night
// cells from the back; one atomic per warp and class for the threads that
// arrive together
__device__ __forceinline__ void nt_enqueue(const Params& P, int cell, bool day) {
    const unsigned act = __activemask();
    const unsigned lane = threadIdx.x & 31u, below = (1u << lane) - 1u;
    const unsigned dm = __ballot_sync(act, day), nm = act & ~dm;
    const int leader = __ffs(act) - 1;
    int dbase = 0, nbase = 0;
    if ((int)lane == leader) {
        if (dm) dbase = atomicAdd(P.nt_head + 1, __popc(dm));
        if (nm) nbase = atomicAdd(P.nt_head + 2, __popc(nm));
    }
    dbase = __shfl_sync(act, dbase, leader);
    nbase = __shfl_sync(act, nbase, leader);
    if (day)
        P.nt_list[dbase + __popc(dm & below)] = cell;
    else
        P.nt_list[P.nt_qcap - 1 - (nbase + __popc(nm & below))] = cell;
}

// the plain start of a cell from its record: P.npass_plain reference passes
// from the start state (ck0 from the record, cc from hc) -> x; the cell
// enters the work queue (day cells from the front, night cells from the
// back). MODE 0: every cell; MODE 2: only cells whose FP32 start
// (k_nt_start32) was not finite (stat < 0); MODE 3 (learned restart): the
// cells of the slots that k_nt_collect filled, with the network's features
// of the plain start at the cell's slot.
template <int MODE>
__global__ void __launch_bounds__(128) k_nt_start(Params P) {
    static_assert(MODE == 0 || MODE == 2 || MODE == 3, "start modes");
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    int cell;
    if (MODE == 3) {  // thread t: slot t (k_nt_collect)
        if (t >= min(P.nt_head[3], P.mlp_cap)) return;
        cell = P.mlp_cells[t];
    } else {
        if (t >= P.win_ncell) return;
        cell = win_cell(P, t);
        if (MODE == 2 && P.nt_stat[cell] >= 0) return;
    }
    const int slot = t;
    const double* r = P.nt_rec + (size_t)cell * NT_REC;
    CellFix F;
    F.o2 = r[NT_RF]; F.n2 = r[NT_RF + 1]; F.h2 = r[NT_RF + 2]; F.co2 = r[NT_RF + 3]; F.hnm = r[NT_RF + 4];
    F.parthno3 = r[NT_RF + 5]; F.parth2o = r[NT_RF + 6]; F.parthcl = r[NT_RF + 7]; F.parthbr = r[NT_RF + 8];
    F.rain_hno3 = r[NT_RF + 9]; F.rain_hno4 = 0.; F.rain_hcl = r[NT_RF + 10]; F.rain_hbr = r[NT_RF + 11];
    F.rain_h2o2 = r[NT_RF + 12]; F.rain_ch2o = 0.; F.rain_ch3o2h = 0.;
    F.sza = r[NT_RSZA];
    const size_t g = cell_global(P, cell), pl = plane3(P);
    double K[NRATE], tj[NPHOT], het[9], ck0[NBCON], ck[NBCON], cc[NCM];
#pragma unroll
    for (int n = 0; n < NRATE; n++) K[n] = r[NT_RK + n];
#pragma unroll
    for (int n = 0; n < NPHOT; n++) tj[n] = r[NT_RJ + n];
#pragma unroll
    for (int n = 0; n < 9; n++) het[n] = r[NT_RH + n];
#pragma unroll
    for (int n = 0; n < NBCON; n++) ck[n] = ck0[n] = r[NT_RCK0 + n];
#pragma unroll
    for (int n = 0; n < NCM; n++) cc[n] = P.hc[g + pl * n] * F.hnm;
#pragma unroll 1
    for (int it = 0; it < P.npass_plain; it++) cell_pass(F, K, tj, het, ck0, P.sc.dt, ck, cc);
    double* x = P.nt_x + (size_t)cell * NT_NX;
#pragma unroll
    for (int n = 0; n < NBCON - 1; n++) x[n] = ck[n];
#pragma unroll
    for (int n = 0; n < NCM; n++) x[NBCON - 1 + n] = cc[n];
    if (MODE == 3) {
        float fe[64];
        cell_features(P, g, F.hnm, F.sza, r[NT_RSURF], ck, cc, fe);
        float4* o = reinterpret_cast<float4*>(P.mlp_feat + (size_t)slot * 64);
#pragma unroll
        for (int i = 0; i < 16; i++) o[i] = make_float4(fe[4 * i], fe[4 * i + 1], fe[4 * i + 2], fe[4 * i + 3]);
        atomicAdd(P.nonfinite + 4, 1ULL);
    }
    P.nt_stat[cell] = 0;
    nt_enqueue(P, cell, F.sza <= 95.);
    if (MODE == 2) atomicAdd(P.nonfinite + 6, 1ULL);
}

// the plain start of the mixed solver: the same P.npass_plain reference passes
// in FP32 arithmetic, from the FP32 record (rates, fixed quantities) and the
// start state rounded to FP32. The start only seeds Newton, whose FP64
// residual and update decide the converged answer. The day/night branch
// follows the FP64 zenith angle. A cell whose FP32 start is not finite (a
// night-time NO2/NO3 ratio beyond the FP32 range) gets stat -1 and is started
// again in FP64 by k_nt_start<2>; the others enter the work queue.
// MODE 0: every cell of the window; MODE 3 (learned restart): the cells of
// the slots that k_nt_collect filled, with the network's features of the
// plain start at the cell's slot (a cell whose FP32 start is not finite keeps
// stat -1 and falls back).
template <int MODE>
__global__ void __launch_bounds__(128) k_nt_start32(Params P) {
    static_assert(MODE == 0 || MODE == 3, "start modes");
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    int cell;
    if (MODE == 3) {
        if (t >= min(P.nt_head[3], P.mlp_cap)) return;
        cell = P.mlp_cells[t];
    } else {
        if (t >= P.win_ncell) return;
        cell = win_cell(P, t);
    }
    const double* r = P.nt_rec + (size_t)cell * NT_REC;
    const float* q = P.nt_rec32 + (size_t)cell * NT_REC32;
    const double hnm = r[NT_RF + 4];
    const bool day = r[NT_RSZA] <= 95.;
    CellFixT<float> F;
    F.o2 = q[NT_RF]; F.n2 = q[NT_RF + 1]; F.h2 = q[NT_RF + 2]; F.co2 = q[NT_RF + 3]; F.hnm = q[NT_RF + 4];
    F.parthno3 = q[NT_RF + 5]; F.parth2o = q[NT_RF + 6]; F.parthcl = q[NT_RF + 7]; F.parthbr = q[NT_RF + 8];
    F.rain_hno3 = q[NT_RF + 9]; F.rain_hno4 = 0.f; F.rain_hcl = q[NT_RF + 10]; F.rain_hbr = q[NT_RF + 11];
    F.rain_h2o2 = q[NT_RF + 12]; F.rain_ch2o = 0.f; F.rain_ch3o2h = 0.f;
    F.sza = day ? 0.f : 180.f;  // only the day/night test reads it, decided in FP64
    const size_t g = cell_global(P, cell), pl = plane3(P);
    float K[NRATE], tj[NPHOT], het[9], ck0[NBCON], ck[NBCON], cc[NCM];
#pragma unroll
    for (int n = 0; n < NRATE; n++) K[n] = q[NT_RK + n];
#pragma unroll
    for (int n = 0; n < NPHOT; n++) tj[n] = q[NT_RJ + n];
#pragma unroll
    for (int n = 0; n < 9; n++) het[n] = q[NT_RH + n];
    // double <-> float by integer operations (newton_num.cuh): a conversion
    // instruction would issue on the FP64 pipe
#pragma unroll
    for (int n = 0; n < NBCON; n++) ck[n] = ck0[n] = nt_cvt<float>(r[NT_RCK0 + n]);
#pragma unroll
    for (int n = 0; n < NCM; n++) cc[n] = nt_cvt<float>(P.hc[g + pl * n] * hnm);
    const float dt = nt_cvt<float>(P.sc.dt);
#pragma unroll 1
    for (int it = 0; it < P.npass_plain; it++) cell_pass(F, K, tj, het, ck0, dt, ck, cc);
    bool finite = true;
#pragma unroll
    for (int n = 0; n < NBCON - 1; n++) finite &= isfinite(ck[n]);
#pragma unroll
    for (int n = 0; n < NCM; n++) finite &= isfinite(cc[n]);
    if (!finite) {
        P.nt_stat[cell] = -1;
        return;
    }
    double* x = P.nt_x + (size_t)cell * NT_NX;
    double xd[NT_NX];
#pragma unroll
    for (int n = 0; n < NBCON - 1; n++) x[n] = xd[n] = nt_widen(ck[n]);
#pragma unroll
    for (int n = 0; n < NCM; n++) x[NBCON - 1 + n] = xd[NBCON - 1 + n] = nt_widen(cc[n]);
    if (MODE == 3) {
        double ckd[NBCON];
#pragma unroll
        for (int n = 0; n < NBCON - 1; n++) ckd[n] = xd[n];
        ckd[NBCON - 1] = 0.;
        float fe[64];
        cell_features(P, g, hnm, r[NT_RSZA], r[NT_RSURF], ckd, xd + NBCON - 1, fe);
        float4* o = reinterpret_cast<float4*>(P.mlp_feat + (size_t)t * 64);
#pragma unroll
        for (int i = 0; i < 16; i++) o[i] = make_float4(fe[4 * i], fe[4 * i + 1], fe[4 * i + 2], fe[4 * i + 3]);
        atomicAdd(P.nonfinite + 4, 1ULL);
    }
    P.nt_stat[cell] = 0;
    nt_enqueue(P, cell, day);
}

// learned restart: each cell of the window whose Newton iteration missed
// (stat < 0) takes a slot k < P.mlp_cap (cells beyond the last slot get stat
// NT_STAT_NOSLOT and fall back); P.nt_head[3] counts the cells that asked
__global__ void __launch_bounds__(128) k_nt_collect(Params P) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P.win_ncell) return;
    const int cell = win_cell(P, t);
    if (P.nt_stat[cell] >= 0) return;
    const int slot = atomicAdd(P.nt_head + 3, 1);
    if (slot < P.mlp_cap)
        P.mlp_cells[slot] = cell;
    else
        P.nt_stat[cell] = NT_STAT_NOSLOT;
}

// learned restart: x_i = max(x_i, 1e-30 hnm) 10^y_i for the cell of each
// slot, y from the network's prediction for that slot. Consecutive threads
// touch consecutive words of a slot's prediction and of its cell's iterate.
// An inference that gave up (its error flag set) left no predictions: every
// cell keeps its plain start and counter 7 records the timeout for the host.
__global__ void __launch_bounds__(128) k_nt_warm(Params P) {
    const bool failed = P.mlp_err && *P.mlp_err != 0u;
    if (failed) {
        if (blockIdx.x == 0 && threadIdx.x == 0) P.nonfinite[7] = 1ULL;
        return;
    }
    const int ns = min(P.nt_head[3], P.mlp_cap);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ns * NT_NX; e += gridDim.x * blockDim.x) {
        const int k = e / NT_NX, i = e - k * NT_NX;
        const size_t cell = (size_t)P.mlp_cells[k];
        const double hnm = P.nt_rec[cell * NT_REC + NT_RF + 4];
        double* x = P.nt_x + cell * NT_NX + i;
        const float yi = fminf(fmaxf(P.mlp_y[(size_t)k * 64 + i], -30.f), 30.f);
        *x = fmax(*x, 1e-30 * hnm) * nt_widen(exp10f(yi));
    }
}

// REF5 in two kernels (k_nt_setup<false>, then this one): the reference's
// P.niter passes from the cell's record (rates, fixed constants, zenith
// angle, ck0) and hc, write-back and (fused) conserv + clamps -- the same
// arithmetic as k_chem, split so that each program is smaller for the
// instruction cache
__global__ void __launch_bounds__(128) k_ref_passes(Params P) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool own = t < P.ncell;  // else: the passes on a valid cell, between the barriers, and no write
    const int cell = own ? t : P.ncell - 1;
    const double* r = P.nt_rec + (size_t)cell * NT_REC;
    CellPro C;
    C.g = cell_global(P, cell);
    CellFix& F = C.F;
    F.o2 = r[NT_RF]; F.n2 = r[NT_RF + 1]; F.h2 = r[NT_RF + 2]; F.co2 = r[NT_RF + 3]; F.hnm = r[NT_RF + 4];
    F.parthno3 = r[NT_RF + 5]; F.parth2o = r[NT_RF + 6]; F.parthcl = r[NT_RF + 7]; F.parthbr = r[NT_RF + 8];
    F.rain_hno3 = r[NT_RF + 9]; F.rain_hno4 = 0.; F.rain_hcl = r[NT_RF + 10]; F.rain_hbr = r[NT_RF + 11];
    F.rain_h2o2 = r[NT_RF + 12]; F.rain_ch2o = 0.; F.rain_ch3o2h = 0.;
    F.sza = r[NT_RSZA];
    const size_t pl = plane3(P);
    double ck[NBCON], cc[NCM];
#pragma unroll
    for (int n = 0; n < NRATE; n++) C.K[n] = r[NT_RK + n];
#pragma unroll
    for (int n = 0; n < NPHOT; n++) C.tj[n] = r[NT_RJ + n];
#pragma unroll
    for (int n = 0; n < 9; n++) C.A.het[n] = r[NT_RH + n];
#pragma unroll
    for (int n = 0; n < NBCON; n++) ck[n] = C.ck0[n] = r[NT_RCK0 + n];
#pragma unroll
    for (int n = 0; n < NCM; n++) cc[n] = P.hc[C.g + pl * n] * F.hnm;
    // the block's warps run each pass between the same barriers (REF5 at cfg1
    // 40.5 -> 39.2 ms; the same in the Newton starts measured no gain)
#pragma unroll 1
    for (int it = 0; it < P.niter; it++) {
        cell_pass(F, C.K, C.tj, C.A.het, C.ck0, P.sc.dt, ck, cc);
        __syncthreads();
    }
    if (!own) return;
    cell_epilogue(P, C, ck, cc);
}

// the write-back of one cell's Newton answer (mixing ratios, fused conserv
// and clamps); cells the solver handed to its fallback (stat <= 0) are left
// to k_nt_fallback, so that this common path stays small
__device__ __forceinline__ void nt_cell_fix(const double* r, CellFix& F) {
    const double* f = r + NT_RF;
    F.o2 = f[0]; F.n2 = f[1]; F.h2 = f[2]; F.co2 = f[3]; F.hnm = f[4]; F.parthno3 = f[5];
    F.parth2o = f[6]; F.parthcl = f[7]; F.parthbr = f[8]; F.rain_hno3 = f[9];
    F.rain_hno4 = 0.; F.rain_hcl = f[10]; F.rain_hbr = f[11]; F.rain_h2o2 = f[12];
    F.rain_ch2o = 0.; F.rain_ch3o2h = 0.;
    F.sza = r[NT_RSZA];
}

// MODE 0: the cells of the window that converged from the plain start
// (0 < stat < NT_RESTART_BIAS); MODE 1: the cells of the learned restart's
// slots that converged in its solve (stat >= NT_RESTART_BIAS), after
// k_nt_fallback<2> wrote the fallback answer of every slot. MODE 0 touches
// none of the restart's cells and reads no status its solve may still
// change, so it may run while the restart is in flight.
template <int MODE>
__global__ void __launch_bounds__(128) k_nt_finish(Params P) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    bool own;
    int cell = 0;
    if (MODE == 0) {
        own = t < P.win_ncell;
        if (own) cell = win_cell(P, t);
    } else {
        own = t < min(P.nt_head[3], P.mlp_cap);
        if (own) cell = P.mlp_cells[t];
    }
    const int stat = own ? P.nt_stat[cell] : 0;
    const int lo = MODE == 0 ? 0 : NT_RESTART_BIAS, hi = MODE == 0 ? NT_RESTART_BIAS : INT_MAX;
    const bool mine = stat > lo && stat < hi;
    // a restarted cell that missed again keeps the fallback answer written for
    // it (whose non-finite values, if any, are counted here)
    if (MODE == 1 && own && !mine) {
        atomicAdd(P.nonfinite + 2, 1ULL);
        if (P.check) {
            const size_t g = cell_global(P, cell), pl = plane3(P);
            unsigned int bad = 0;
            for (int n = 0; n < NBCON; n++) bad += !isfinite(P.qj1[g + pl * n]);
            for (int n = 0; n < NCM; n++) bad += !isfinite(P.hc[g + pl * n]);
            if (bad) atomicAdd(P.nonfinite, (unsigned long long)bad);
        }
    }
    // iteration statistics, one atomic per warp (blocks are whole warps)
    const unsigned it = mine ? (unsigned)(stat - lo) : 0u;
    const unsigned sum = __reduce_add_sync(0xffffffffu, it), most = __reduce_max_sync(0xffffffffu, it);
    if ((threadIdx.x & 31u) == 0 && sum) {
        atomicAdd(P.nonfinite + 1, (unsigned long long)sum);
        atomicMax(P.nonfinite + 3, (unsigned long long)most);
    }
    if (!mine) return;
    const double* r = P.nt_rec + (size_t)cell * NT_REC;
    const double* x = P.nt_x + (size_t)cell * NT_NX;
    CellPro C;
    C.g = cell_global(P, cell);
    nt_cell_fix(r, C.F);
    double ck[NBCON], cc[NCM];
#pragma unroll
    for (int n = 0; n < NBCON - 1; n++) ck[n] = x[n];
    ck[NBCON - 1] = r[NT_RCK0 + NBCON - 1];
#pragma unroll
    for (int n = 0; n < NCM; n++) cc[n] = x[NBCON - 1 + n];
    cell_epilogue<true>(P, C, ck, cc);
}

// fallback of the cells the Newton solver did not converge: the reference
// scheme's niter passes from the start state, then the write-back.
// MODE 0: the cells of the window with stat <= 0 (no learned restart);
// MODE 1: those with stat NT_STAT_NOSLOT (the restart had no slot for them);
// MODE 2: every cell of the restart's slots, ahead of their second solve and
// beside it: k_nt_finish<1> then writes back the ones it converged over
// these answers and counts the others as fallbacks.
template <int MODE>
__global__ void __launch_bounds__(128) k_nt_fallback(Params P) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    int cell;
    if (MODE == 2) {
        if (t >= min(P.nt_head[3], P.mlp_cap)) return;
        cell = P.mlp_cells[t];
    } else {
        if (t >= P.win_ncell) return;
        cell = win_cell(P, t);
        const int stat = P.nt_stat[cell];
        if (MODE == 0 ? stat > 0 : stat != NT_STAT_NOSLOT) return;
    }
    const double* r = P.nt_rec + (size_t)cell * NT_REC;
    CellPro C;
    C.g = cell_global(P, cell);
    CellFix& F = C.F;
    nt_cell_fix(r, F);
    const size_t pl = plane3(P);
    double ck[NBCON], cc[NCM];
#pragma unroll
    for (int n = 0; n < NBCON; n++) C.ck0[n] = r[NT_RCK0 + n];
#pragma unroll
    for (int n = 0; n < NRATE; n++) C.K[n] = r[NT_RK + n];
#pragma unroll
    for (int n = 0; n < NPHOT; n++) C.tj[n] = r[NT_RJ + n];
#pragma unroll
    for (int n = 0; n < 9; n++) C.A.het[n] = r[NT_RH + n];
#pragma unroll
    for (int n = 0; n < NBCON; n++) ck[n] = C.ck0[n];
#pragma unroll
    for (int n = 0; n < NCM; n++) cc[n] = P.hc[C.g + pl * n] * F.hnm;
#pragma unroll 1
    for (int it = 0; it < P.niter; it++) cell_pass(F, C.K, C.tj, C.A.het, C.ck0, P.sc.dt, ck, cc);
    if (MODE != 2) atomicAdd(P.nonfinite + 2, 1ULL);
    cell_epilogue<true>(P, C, ck, cc);
}

// ----------------------------------------------------------------------------
// k_tail — levels nivbas+1..niv of the rows: clamps F:431-440, HNO3 gas F:444-450
// ----------------------------------------------------------------------------
__global__ void k_tail(Params P) {
    const long long n = (long long)P.nlon * P.win_nr * (P.niv - P.nivbas);
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n) return;
    const int i = (int)(idx % P.nlon);
    const long long rest = idx / P.nlon;
    const int j = P.ilat0 + P.win_r0 + (int)(rest % P.win_nr);
    const int k = P.nivbas + (int)(rest / P.win_nr);
    const size_t g = (size_t)i + (size_t)P.nlon * ((size_t)j + (size_t)P.nlat * k);
    const size_t pl = plane3(P);
#pragma unroll 6
    for (int s = 0; s < NBCON - 1; s++) P.qj1[g + pl * s] = clamp_1e30(P.qj1[g + pl * s]);
    P.qj1[g + pl * (NBCON - 1)] = P.qj1[g + pl * 4];
}

// ----------------------------------------------------------------------------
// k_conserv — standalone conserv + clamps on rows, all levels
// ----------------------------------------------------------------------------
__global__ void k_conserv(Params P) {
    const long long n = (long long)P.nlon * P.nrows * P.niv;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n) return;
    const int i = (int)(idx % P.nlon);
    const long long rest = idx / P.nlon;
    const int j = P.ilat0 + (int)(rest % P.nrows);
    const int k = (int)(rest / P.nrows);
    const size_t g = (size_t)i + (size_t)P.nlon * ((size_t)j + (size_t)P.nlat * k);
    const size_t pl = plane3(P);
    double q[NBCON], h[NCM];
#pragma unroll
    for (int s = 0; s < NBCON; s++) q[s] = P.qj1[g + pl * s];
    if (k < P.nivbas) {
#pragma unroll
        for (int s = 0; s < NCM; s++) h[s] = P.hc[g + pl * s];
        cell_conserv(q, h);
#pragma unroll
        for (int s = 0; s < NCM; s++) P.hc[g + pl * s] = h[s];
    }
#pragma unroll
    for (int s = 0; s < NBCON - 1; s++) q[s] = clamp_1e30(q[s]);
    if (k >= P.nivbas) q[NBCON - 1] = q[4];
#pragma unroll
    for (int s = 0; s < NBCON; s++) P.qj1[g + pl * s] = q[s];
}

// ----------------------------------------------------------------------------
// handle
// ----------------------------------------------------------------------------
struct Handle {
    int nlon, nlat, niv, nivbas, nivhau, nrappmax, niter, flags;
    int device;
    int solver = REPROBUS_SOLVER_REF5;  // which kernel integrates the cells
    int npass = 5, maxit = 12;          // Newton: reference passes before, iteration cap
    double tol = 1e-4;                  // Newton: scaled step tolerance
    double troe[18];
    double* d_ajl = nullptr;
    double* d_o3up = nullptr;
    double* d_col = nullptr;
    unsigned long long* d_count = nullptr;
    cudaStream_t own = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t ev2 = nullptr, ev3 = nullptr;  // around the persistent solve kernel (stats.solve_ms)
    cudaEvent_t ev4 = nullptr, ev5 = nullptr;  // around a second solve (host-array entry point)
    // the learned restart runs on its own stream of the highest priority
    // while the handle's stream writes back the converged cells
    cudaStream_t rstream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_collect = nullptr, ev_spec = nullptr;
    // device mirrors for the host-pointer entry point (allocated on first use)
    double* m_alt = nullptr;
    double* m_traj[4] = {nullptr, nullptr, nullptr, nullptr};
    double* m_qj1 = nullptr;
    double* m_hc = nullptr;
    double* m_out[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};  // vsed, parth2o, parthno3, sza3d, surfarea
    // Newton pipeline buffers (allocated when a Newton solver is selected)
    double* nt_rec = nullptr;
    float* nt_rec32 = nullptr;
    double* nt_x = nullptr;
    int* nt_stat = nullptr;
    int* nt_list = nullptr;
    int* nt_head = nullptr;
    int nsm = 0;
    // persistent solve kernel shape per matrix precision ([0] FP32, [1] FP64)
    int want_lanes = 0, want_bps = 0, want_zs = 0;   // reprobus_chem_set_tuning; lanes 0: autotune
    const NtVariant* nt_var[2] = {nullptr, nullptr};
    int nt_bps[2] = {0, 0};
    // the learned restart's solve: a few hundred cells, so the form with the
    // shortest iteration (4 warps per cell) rather than the autotuned one
    const NtVariant* rs_var[2] = {nullptr, nullptr};
    // REF5 as the rate-stage kernel + the passes kernel through the cell
    // records (false: the single kernel k_chem, no record buffers)
    bool split_ref5 = true;
    // CUDA graph of the step (REPROBUS_USE_GRAPH)
    cudaGraphExec_t gexec = nullptr;
    int gexec_sig = -1;
    unsigned graph_ready = 0;  // configurations that have run once directly
    // learned restart (reprobus_chem_set_mlp): the network and the buffers of
    // its mlp_cap slots (features, predictions, cells)
    void* mlp = nullptr;
    int mlp_cap = 0;
    float* mlp_feat = nullptr;
    float* mlp_y = nullptr;
    int* mlp_cells = nullptr;
    // host-array entry point: copy streams and events of its row chunks
    cudaStream_t cin = nullptr, cout = nullptr;
    cudaEvent_t ev_in[4] = {}, ev_comp[4] = {};
    // scratch of the column-physics entry points (column_kernels.cu)
    void* col_scratch = nullptr;
    size_t col_scratch_bytes = 0;
};

static const char* kVersion = "reprobus_gb300 0.1 (sm_103a, FP64 reference scheme)";

extern "C" const char* reprobus_version(void) { return kVersion; }
extern "C" const char* reprobus_last_error(void) { return g_err; }

extern "C" int reprobus_chem_troe(double* troe) {
    if (!troe) return set_err(REPROBUS_ERR_ARG, "troe is NULL");
    troe[0] = 4.4e-32 * pow(300., 1.3);
    troe[1] = 7.5e-11 * pow(300., -0.2);
    troe[2] = 2.0e-30 * pow(300., 4.4);
    troe[3] = 1.4e-12 * pow(300., 0.7);
    troe[4] = 1.8e-30 * pow(300., 3.0);
    troe[5] = 2.8e-11 * pow(300., 0.0);
    troe[6] = 2.0e-31 * pow(300., 3.4);
    troe[7] = 2.9e-12 * pow(300., 1.1);
    troe[8] = 1.8e-31 * pow(300., 3.4);
    troe[9] = 1.5e-11 * pow(300., 1.9);
    troe[10] = 1.8e-31 * pow(300., 2.0);
    troe[11] = 1.0e-10 * pow(300., 1.0);
    troe[12] = 1.6e-32 * pow(300., 4.5);
    troe[13] = 3.0e-12 * pow(300., 2.0);
    troe[14] = 5.2e-31 * pow(300., 3.2);
    troe[15] = 6.9e-12 * pow(300., 2.9);
    troe[16] = 4.0e-31 * pow(300., 3.6);
    troe[17] = 1.2e-12 * pow(300., -1.1);
    return REPROBUS_OK;
}

static void free_handle(Handle* h) {
    if (!h) return;
    cudaFree(h->d_ajl);
    cudaFree(h->d_o3up);
    cudaFree(h->d_col);
    cudaFree(h->d_count);
    cudaFree(h->m_alt);
    for (auto& p : h->m_traj) cudaFree(p);
    cudaFree(h->m_qj1);
    cudaFree(h->m_hc);
    for (auto& p : h->m_out) cudaFree(p);
    cudaFree(h->nt_rec);
    cudaFree(h->nt_rec32);
    cudaFree(h->nt_x);
    cudaFree(h->nt_stat);
    cudaFree(h->nt_list);
    cudaFree(h->nt_head);
    cudaFree(h->mlp_feat);
    cudaFree(h->mlp_y);
    cudaFree(h->mlp_cells);
    cudaFree(h->col_scratch);
    for (int c = 0; c < 4; c++) {
        if (h->ev_in[c]) cudaEventDestroy(h->ev_in[c]);
        if (h->ev_comp[c]) cudaEventDestroy(h->ev_comp[c]);
    }
    if (h->cin) cudaStreamDestroy(h->cin);
    if (h->cout) cudaStreamDestroy(h->cout);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    if (h->ev2) cudaEventDestroy(h->ev2);
    if (h->ev3) cudaEventDestroy(h->ev3);
    if (h->ev4) cudaEventDestroy(h->ev4);
    if (h->ev5) cudaEventDestroy(h->ev5);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_collect) cudaEventDestroy(h->ev_collect);
    if (h->ev_spec) cudaEventDestroy(h->ev_spec);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    if (h->rstream) cudaStreamDestroy(h->rstream);
    if (h->own) cudaStreamDestroy(h->own);
    delete h;
}

// The rate stage takes ln of the 18 Troe prefactors (COMMON /constant/,
// :5927-5948): each must be positive and finite, as the reference's are.
static int check_troe(const double* troe) {
    for (int i = 0; i < 18; i++)
        if (!(troe[i] > 0.) || !(troe[i] < INFINITY))
            return set_err(REPROBUS_ERR_ARG, "troe[%d] = %g: the Troe prefactors must be positive and finite", i,
                           troe[i]);
    return REPROBUS_OK;
}

extern "C" int reprobus_chem_init(const double* ajl, const double* o3up, const double* troe, int nlon, int nlat,
                                  int niv, int nivbas, int nivhau, int nrappmax, int niter, int flags,
                                  void** handle) {
    if (!handle) return set_err(REPROBUS_ERR_ARG, "handle is NULL");
    *handle = nullptr;
    if (!ajl || !o3up || !troe) return set_err(REPROBUS_ERR_ARG, "ajl, o3up and troe must be non-NULL");
    if (int rc = check_troe(troe)) return rc;
    if (nlon <= 0 || nlat <= 0 || niv <= 0 || nivbas <= 0 || nivbas > niv || nivhau < 1 || nivhau > nivbas ||
        nrappmax <= 0 || niter < 0)
        return set_err(REPROBUS_ERR_ARG, "bad sizes: nlon=%d nlat=%d niv=%d nivbas=%d nivhau=%d nrappmax=%d niter=%d",
                       nlon, nlat, niv, nivbas, nivhau, nrappmax, niter);
    if ((long long)nlon * nlat * nivbas >= (1LL << 30))
        return set_err(REPROBUS_ERR_ARG, "grid too large for 32-bit cell indexing");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return set_err(REPROBUS_ERR_NODEVICE, "no CUDA device visible");
    Handle* h = new (std::nothrow) Handle();
    if (!h) return set_err(REPROBUS_ERR_ARG, "out of host memory");
    h->nlon = nlon;
    h->nlat = nlat;
    h->niv = niv;
    h->nivbas = nivbas;
    h->nivhau = nivhau;
    h->nrappmax = nrappmax;
    h->niter = niter;
    h->flags = flags;
    memcpy(h->troe, troe, sizeof(h->troe));
    int rc = REPROBUS_OK;
    auto fail = [&](int code) {
        free_handle(h);
        return code;
    };
    cudaError_t e;
    if ((e = cudaGetDevice(&h->device)) != cudaSuccess) return fail(set_err(REPROBUS_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e)));
    const size_t najl = (size_t)(NPHOT - 1) * NZ * NSZA * NOZO;
    const size_t ncell = (size_t)nlon * nlat * nivbas;
    const size_t ncol = (size_t)nlon * nlat;
    if ((e = cudaStreamCreateWithFlags(&h->own, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreate(&h->ev0)) != cudaSuccess || (e = cudaEventCreate(&h->ev1)) != cudaSuccess ||
        (e = cudaEventCreate(&h->ev2)) != cudaSuccess || (e = cudaEventCreate(&h->ev3)) != cudaSuccess ||
        (e = cudaEventCreate(&h->ev4)) != cudaSuccess || (e = cudaEventCreate(&h->ev5)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&h->ev_collect, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&h->ev_spec, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaMalloc(&h->d_ajl, najl * sizeof(double))) != cudaSuccess ||
        (e = cudaMalloc(&h->d_o3up, 80 * sizeof(double))) != cudaSuccess ||
        (e = cudaMalloc(&h->d_col, (3 * ncell + ncol) * sizeof(double))) != cudaSuccess ||
        (e = cudaMalloc(&h->d_count, 8 * sizeof(unsigned long long))) != cudaSuccess ||
        (e = cudaMemcpy(h->d_ajl, ajl, najl * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(h->d_o3up, o3up, 80 * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess)
        return fail(set_err(REPROBUS_ERR_CUDA, "init: %s", cudaGetErrorString(e)));
    h->stream = h->own;
    (void)rc;
    *handle = h;
    return REPROBUS_OK;
}

namespace rpb {
__attribute__((visibility("hidden"))) int handle_info(void* handle, HandleInfo* out) {
    const Handle* h = (const Handle*)handle;
    if (!h) return set_err(REPROBUS_ERR_ARG, "handle is NULL");
    out->device = h->device;
    out->nlon = h->nlon;
    out->nlat = h->nlat;
    out->niv = h->niv;
    out->nivbas = h->nivbas;
    out->nivhau = h->nivhau;
    out->nrappmax = h->nrappmax;
    out->stream = h->stream;
    return REPROBUS_OK;
}

__attribute__((visibility("hidden"))) int handle_scratch(void* handle, size_t bytes, void** out) {
    Handle* h = (Handle*)handle;
    if (!h) return set_err(REPROBUS_ERR_ARG, "handle is NULL");
    if (h->col_scratch_bytes < bytes) {
        CUDA_TRY(cudaStreamSynchronize(h->stream));
        cudaFree(h->col_scratch);
        h->col_scratch = nullptr;
        h->col_scratch_bytes = 0;
        CUDA_TRY(cudaMalloc(&h->col_scratch, bytes));
        h->col_scratch_bytes = bytes;
    }
    *out = h->col_scratch;
    return REPROBUS_OK;
}
}  // namespace rpb

extern "C" int reprobus_chem_free(void* handle) {
    free_handle((Handle*)handle);
    return REPROBUS_OK;
}

extern "C" int reprobus_chem_set_stream(void* handle, void* stream) {
    Handle* h = (Handle*)handle;
    if (!h) return set_err(REPROBUS_ERR_ARG, "handle is NULL");
    h->stream = stream ? (cudaStream_t)stream : h->own;
    return REPROBUS_OK;
}

// per-step zenith constants, zenith F:5338-5380 (host, once per call)
static void step_const(const Handle* h, double day, double dt, StepConst& sc) {
    const double pi = PI;
    double ut = (day - trunc(day)) * 24.;
    double tz = 2. * pi * day / 365.;
    double sintz = sin(tz);
    double costz = cos(tz);
    double sin2tz = 2. * sintz * costz;
    double cos2tz = costz * costz - sintz * sintz;
    double sin3tz = sintz * cos2tz + costz * sin2tz;
    double cos3tz = costz * cos2tz - sintz * sin2tz;
    double rdecl = 0.006918 - 0.399912 * costz + 0.070257 * sintz - 0.006758 * cos2tz + 0.000907 * sin2tz -
                   0.002697 * cos3tz + 0.001480 * sin3tz;
    double eqr = 0.000075 + 0.001868 * costz - 0.032077 * sintz - 0.014615 * cos2tz - 0.040849 * sin2tz;
    sc.ut = ut;
    sc.eqh = eqr * 24. / (2. * pi);
    sc.srd = sin(rdecl);
    sc.crd = cos(rdecl);
    sc.dt = dt;
    memcpy(sc.troe, h->troe, sizeof(sc.troe));
    for (int i = 0; i < 18; i++) sc.ltroe[i] = sc.troe[i] > 0. ? log(sc.troe[i]) : 0.;
}

static int check_rows(const Handle* h, int ilat0, int ilat1) {
    if (ilat0 < 1 || ilat1 > h->nlat || ilat0 > ilat1)
        return set_err(REPROBUS_ERR_ARG, "bad row range %d..%d (nlat=%d)", ilat0, ilat1, h->nlat);
    return REPROBUS_OK;
}

static void fill_params(const Handle* h, Params& P, int ilat0, int ilat1) {
    memset(&P, 0, sizeof(P));
    P.nlon = h->nlon;
    P.nlat = h->nlat;
    P.niv = h->niv;
    P.nivbas = h->nivbas;
    P.nivhau = h->nivhau;
    P.ilat0 = ilat0 - 1;
    P.nrows = ilat1 - ilat0 + 1;
    P.niter = h->niter;
    P.ncol = h->nlon * P.nrows;
    P.ncell = P.ncol * h->nivbas;
    P.win_r0 = 0;
    P.win_nr = P.nrows;
    P.win_ncol = P.ncol;
    P.win_ncell = P.ncell;
    P.nt_qcap = P.ncell;
    P.ajl = h->d_ajl;
    P.o3up = h->d_o3up;
    P.col = h->d_col;
    P.nonfinite = h->d_count;
    P.npass = h->npass;
    P.maxit = h->maxit;
    P.tol = h->tol;
}

// every compiled solve-kernel variant of one matrix precision
static int nt_all_variants(bool mixed, const NtVariant** out, int cap) {
    int n = 0, k = 0;
    const NtVariant* lists[6] = {};
    int counts[6] = {0, 0, 0, 0, 0, 0};
    const int nl = 6;
    if (mixed) {
        lists[0] = nt_variants_f32_zr(&counts[0]);
        lists[1] = nt_variants_f32_zs(&counts[1]);
        lists[2] = nt_variants_f32_pp(&counts[2]);
        lists[3] = nt_variants_f32_sp(&counts[3]);
        lists[4] = nt_variants_f32_ls(&counts[4]);
        lists[5] = nt_variants_f32_wc(&counts[5]);
    } else {
        lists[0] = nt_variants_f64_zr(&counts[0]);
        lists[1] = nt_variants_f64_zs(&counts[1]);
        lists[2] = nt_variants_f64_pp(&counts[2]);
        lists[3] = nt_variants_f64_sp(&counts[3]);
        lists[4] = nt_variants_f64_ls(&counts[4]);
        lists[5] = nt_variants_f64_wc(&counts[5]);
    }
    for (int l = 0; l < nl; l++)
        for (k = 0; k < counts[l] && n < cap; k++) out[n++] = &lists[l][k];
    return n;
}

static int ensure_newton(Handle* h) {
    if (h->nt_x) return REPROBUS_OK;
    const size_t nc = (size_t)h->nlon * h->nlat * h->nivbas;
    CUDA_TRY(cudaMalloc(&h->nt_rec, nc * NT_REC * sizeof(double)));
    CUDA_TRY(cudaMalloc(&h->nt_rec32, nc * NT_REC32 * sizeof(float)));
    CUDA_TRY(cudaMalloc(&h->nt_x, nc * NT_NX * sizeof(double)));
    CUDA_TRY(cudaMalloc(&h->nt_stat, nc * sizeof(int)));
    CUDA_TRY(cudaMalloc(&h->nt_list, nc * sizeof(int)));
    CUDA_TRY(cudaMalloc(&h->nt_head, 8 * sizeof(int)));
    CUDA_TRY(cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, h->device));
    return REPROBUS_OK;
}

// blocks of the fused REF5 kernel k_chem (256 threads in lock-step)
constexpr int SETUP_TB = 256;
// the rate-stage kernel of the Newton pipeline (and of the split REF5): two
// blocks of 512 threads per SM in lock-step. Measured at cfg1 (mixed step):
// without the barriers 61.3 -> 64.7 ms; 128 / 256 / 512 / 1024 threads per
// block at 64 registers: 63.1 / 61.3 / 60.4 / 63.9 ms
constexpr int NT_SETUP_TB = 512;
static void launch_setup(Handle* h, const Params& P, bool mixed) {
    const unsigned nb = (unsigned)((P.win_ncell + NT_SETUP_TB - 1) / NT_SETUP_TB);
    if (mixed)
        k_nt_setup<true, NT_SETUP_TB, true><<<nb, NT_SETUP_TB, 0, h->stream>>>(P);
    else
        k_nt_setup<false, NT_SETUP_TB, true><<<nb, NT_SETUP_TB, 0, h->stream>>>(P);
}

// rate stage and plain start of the cells of P's row window; they join the
// work queue, whose heads the caller has zeroed
static void newton_front(Handle* h, const Params& P, bool mixed) {
    const int tb = 128;
    launch_setup(h, P, mixed);
    if (mixed) {
        k_nt_start32<0><<<(P.win_ncell + tb - 1) / tb, tb, 0, h->stream>>>(P);
        k_nt_start<2><<<(P.win_ncell + tb - 1) / tb, tb, 0, h->stream>>>(P);
    } else {
        k_nt_start<0><<<(P.win_ncell + tb - 1) / tb, tb, 0, h->stream>>>(P);
    }
}

static int enqueue_setup(Handle* h, Params& P, bool mixed) {
    CUDA_TRY(cudaMemsetAsync(h->nt_head, 0, 8 * sizeof(int), h->stream));
    newton_front(h, P, mixed);
    return REPROBUS_OK;
}

// Autotuner of the persistent solve kernel: every compiled shape (lanes per
// block) at every resident block count per SM that fits is timed on this
// step's cells (setup, then the timed solve; the setup restores the iterate
// and the queue between candidates) and the fastest is kept for the handle.
// Persisted choices of the autotuner (REPROBUS_TUNE_CACHE names a text file):
// one line per choice, "<key> <lanes per block> <zshared> <blocks per SM>
// <ms>", the key naming the GPU model, its compute capability and SM count,
// the matrix precision and the step's cell count. The last line of a key
// wins; a line whose shape this build does not have is ignored.
static void tune_key(const Handle* h, bool mixed, int ncell, char* key, size_t n) {
    cudaDeviceProp pr;
    if (cudaGetDeviceProperties(&pr, h->device) != cudaSuccess) memset(&pr, 0, sizeof(pr));
    char name[128];
    snprintf(name, sizeof(name), "%s", pr.name);
    for (char* c = name; *c; c++)
        if (*c == ' ' || *c == '\t') *c = '_';
    snprintf(key, n, "%s_sm%d%d_%dsm_%s_%dcells", name, pr.major, pr.minor, pr.multiProcessorCount,
             mixed ? "fp32" : "fp64", ncell);
}

static bool tune_cache_lookup(const char* path, const char* key, int* nth, int* zs, int* bps) {
    FILE* f = fopen(path, "r");
    if (!f) return false;
    char line[512], k[256];
    bool found = false;
    while (fgets(line, sizeof(line), f)) {
        int a, b, c;
        if (sscanf(line, "%255s %d %d %d", k, &a, &b, &c) == 4 && strcmp(k, key) == 0) {
            *nth = a, *zs = b, *bps = c;
            found = true;
        }
    }
    fclose(f);
    return found;
}

static void tune_cache_store(const char* path, const char* key, int nth, int zs, int bps, float ms) {
    FILE* f = fopen(path, "a");
    if (!f) return;  // a cache that cannot be written only costs the next handle a tuning run
    fprintf(f, "%s %d %d %d %.3f\n", key, nth, zs, bps, ms);
    fclose(f);
}

static int choose_shape(Handle* h, Params& P, bool mixed) {
    const int ip = mixed ? 0 : 1;
    if (h->nt_var[ip]) return REPROBUS_OK;
    const char* cache = h->want_lanes > 0 ? nullptr : getenv("REPROBUS_TUNE_CACHE");
    char key[256] = "";
    if (cache && cache[0]) {
        tune_key(h, mixed, P.ncell, key, sizeof(key));
        int nth = 0, zs = 0, bps = 0;
        if (tune_cache_lookup(cache, key, &nth, &zs, &bps)) {
            const NtVariant* vc[32];
            const int n = nt_all_variants(mixed, vc, 32);
            for (int i = 0; i < n; i++) {
                if (vc[i]->nth != nth || vc[i]->zshared != zs) continue;
                int occ = 0;
                CUDA_TRY(vc[i]->prepare(&occ));
                if (bps < 1 || bps > occ) break;
                h->nt_var[ip] = vc[i];
                h->nt_bps[ip] = bps;
                return REPROBUS_OK;
            }
        }
    }
    const NtVariant* vs[32];
    const int nv = nt_all_variants(mixed, vs, 32);
    struct Cand { const NtVariant* v; int bps; };
    Cand cands[64];
    int nc = 0;
    // a requested shape that this precision does not have: autotune it instead
    bool want = h->want_lanes > 0;
    if (want) {
        bool any = false;
        for (int i = 0; i < nv; i++) any |= vs[i]->nth == h->want_lanes && vs[i]->zshared == h->want_zs;
        want = any;
    }
    for (int i = 0; i < nv; i++) {
        int occ = 0;
        CUDA_TRY(vs[i]->prepare(&occ));
        if (occ < 1) continue;
        if (want) {
            if (vs[i]->nth != h->want_lanes || vs[i]->zshared != h->want_zs) continue;
            const int b = h->want_bps > 0 && h->want_bps < occ ? h->want_bps : occ;
            cands[nc++] = {vs[i], b};
            continue;
        }
        for (int b = 1; b <= occ && nc < 64; b++) cands[nc++] = {vs[i], b};
    }
    if (nc == 0)
        return set_err(REPROBUS_ERR_ARG, "no compiled solve-kernel shape with %d lanes per block fits", h->want_lanes);
    if (nc == 1) {
        h->nt_var[ip] = cands[0].v;
        h->nt_bps[ip] = cands[0].bps;
        return REPROBUS_OK;
    }
    float best = 1e30f;
    int bi = 0;
    const char* verbose = getenv("REPROBUS_TUNE_VERBOSE");  // print every candidate's time to stderr
    // (events ev4/ev5: ev0 marks the start of the step being prepared)
    for (int c = 0; c < nc; c++) {
        int rc = enqueue_setup(h, P, mixed);
        if (rc) return rc;
        CUDA_TRY(cudaEventRecord(h->ev4, h->stream));
        CUDA_TRY(cands[c].v->launch(P, h->nsm * cands[c].bps, h->stream));
        CUDA_TRY(cudaEventRecord(h->ev5, h->stream));
        CUDA_TRY(cudaEventSynchronize(h->ev5));
        float ms = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&ms, h->ev4, h->ev5));
        if (verbose && verbose[0] == '1')
            fprintf(stderr, "reprobus autotune: %s lanes %d zshared %d blocks/SM %d: %.3f ms\n",
                    mixed ? "fp32" : "fp64", cands[c].v->nth, cands[c].v->zshared, cands[c].bps, ms);
        if (ms < best) {
            best = ms;
            bi = c;
        }
    }
    h->nt_var[ip] = cands[bi].v;
    h->nt_bps[ip] = cands[bi].bps;
    if (key[0]) tune_cache_store(cache, key, cands[bi].v->nth, cands[bi].v->zshared, cands[bi].bps, best);
    // the trial solves counted iterations and FP64 redos: the step counts afresh
    CUDA_TRY(cudaMemsetAsync(h->d_count, 0, 8 * sizeof(unsigned long long), h->stream));
    return REPROBUS_OK;
}

// the Newton solvers' buffers and fields of P, and the solve-kernel shape
// (autotuned on P's cells the first time)
static int newton_prepare(Handle* h, Params& P) {
    int rc = ensure_newton(h);
    if (rc) return rc;
    const bool mixed = h->solver == REPROBUS_SOLVER_NEWTON_MIXED;
    P.nt_rec = h->nt_rec;
    P.nt_rec32 = h->nt_rec32;
    P.nt_x = h->nt_x;
    P.nt_stat = h->nt_stat;
    P.nt_list = h->nt_list;
    P.nt_head = h->nt_head;
    P.npass_plain = h->npass;
    if (h->mlp) {
        if (!h->mlp_feat) {
            const long long nc = (long long)h->nlon * h->nlat * h->nivbas;
            h->mlp_cap = (int)(nc < MLP_RESTART_CAP ? nc : MLP_RESTART_CAP);
            CUDA_TRY(cudaMalloc(&h->mlp_feat, (size_t)h->mlp_cap * MLP_FEAT * sizeof(float)));
            CUDA_TRY(cudaMalloc(&h->mlp_y, (size_t)h->mlp_cap * MLP_YOUT * sizeof(float)));
            CUDA_TRY(cudaMalloc(&h->mlp_cells, (size_t)h->mlp_cap * sizeof(int)));
        }
        const int ip = mixed ? 0 : 1;
        if (!h->rs_var[ip]) {
            int n = 0, occ = 0;
            const NtVariant* v = mixed ? nt_variants_f32_wc(&n) : nt_variants_f64_wc(&n);
            for (int i = 0; i < n; i++)
                if (v[i].zshared == 6) h->rs_var[ip] = &v[i];
            if (!h->rs_var[ip]) return set_err(REPROBUS_ERR_CUDA, "no 4-warps-per-cell solve form compiled");
            CUDA_TRY(h->rs_var[ip]->prepare(&occ));
        }
        P.mlp_cap = h->mlp_cap;
        P.mlp_feat = h->mlp_feat;
        P.mlp_y = h->mlp_y;
        P.mlp_cells = h->mlp_cells;
        P.mlp_err = mlp_err_flag(h->mlp);
    }
    return choose_shape(h, P, mixed);
}

// the persistent solve of the cells of P's work queue; e0/e1 recorded around
// it unless null
static int newton_solve(Handle* h, const Params& P, cudaEvent_t e0, cudaEvent_t e1, bool capturing) {
    const int ip = h->solver == REPROBUS_SOLVER_NEWTON_MIXED ? 0 : 1;
    if (e0) CUDA_TRY(capturing ? cudaEventRecordWithFlags(e0, h->stream, cudaEventRecordExternal)
                               : cudaEventRecord(e0, h->stream));
    CUDA_TRY(h->nt_var[ip]->launch(P, h->nsm * h->nt_bps[ip], h->stream));
    if (e1) CUDA_TRY(capturing ? cudaEventRecordWithFlags(e1, h->stream, cudaEventRecordExternal)
                               : cudaEventRecord(e1, h->stream));
    return REPROBUS_OK;
}

// The learned restart of the cells of P's window whose Newton iteration
// missed (after newton_solve on P's queue): P's queue is emptied and refilled
// with those cells (at most mlp_cap slots), each started from the network's
// prediction for its plain start and solved again; k_nt_fallback<2> writes
// the fallback answer of every slot, then k_nt_finish<1> the answer of those
// that converged. The cell counts stay on the device. st: the restart's
// stream; sf: the stream of the slots' fallback (st too: one after the
// other; else the fallback runs on sf beside the second solve, after sf's
// work so far, and h->ev_collect / h->ev_spec order the two streams).
static int newton_restart(Handle* h, const Params& P0, cudaStream_t st, cudaStream_t sf, int* launches) {
    const int tb = 128;
    if (P0.win_ncell <= 0) return REPROBUS_OK;
    Params P = P0;
    P.stat_bias = NT_RESTART_BIAS;
    const int ip = h->solver == REPROBUS_SOLVER_NEWTON_MIXED ? 0 : 1;
    const unsigned nslot = (unsigned)((h->mlp_cap + tb - 1) / tb);
    CUDA_TRY(cudaMemsetAsync(P.nt_head, 0, 4 * sizeof(int), st));
    CUDA_TRY(cudaMemsetAsync(mlp_err_flag(h->mlp), 0, sizeof(unsigned int), st));
    k_nt_collect<<<(P.win_ncell + tb - 1) / tb, tb, 0, st>>>(P);
    if (h->solver == REPROBUS_SOLVER_NEWTON_MIXED)  // the plain start as the first attempt had it
        k_nt_start32<3><<<nslot, tb, 0, st>>>(P);
    else
        k_nt_start<3><<<nslot, tb, 0, st>>>(P);
    // the fallback answers go to the output arrays, whose hc the starts just
    // read as the start state: the fallback only once they are done
    if (sf != st) {
        CUDA_TRY(cudaEventRecord(h->ev_collect, st));
        CUDA_TRY(cudaStreamWaitEvent(sf, h->ev_collect, 0));
    }
    {
        Params PF = P;
        PF.check = 0;  // k_nt_finish<1> counts the non-finite values of the answers that stay
        k_nt_fallback<2><<<nslot, tb, 0, sf>>>(PF);
    }
    if (sf != st) CUDA_TRY(cudaEventRecord(h->ev_spec, sf));
    int rc = mlp_infer(h->mlp, h->mlp_feat, h->mlp_y, h->mlp_cap, st, P.nt_head + 3);
    if (rc) return rc;
    const unsigned nb = (unsigned)((h->mlp_cap * NT_NX + tb - 1) / tb);
    k_nt_warm<<<nb < 2u * h->nsm ? nb : 2u * h->nsm, tb, 0, st>>>(P);
    CUDA_TRY(h->rs_var[ip]->launch(P, h->nsm, st));
    if (sf != st) CUDA_TRY(cudaStreamWaitEvent(st, h->ev_spec, 0));
    k_nt_finish<1><<<nslot, tb, 0, st>>>(P);
    *launches += 7;
    return REPROBUS_OK;
}

// write-back of the cells of P's row window: converged cells, then the
// reference passes for the others
static void newton_back(Handle* h, const Params& P) {
    const int tb = 128;
    k_nt_finish<0><<<(P.win_ncell + tb - 1) / tb, tb, 0, h->stream>>>(P);
    if (h->mlp)  // the restart wrote back its slots' cells
        k_nt_fallback<1><<<(P.win_ncell + tb - 1) / tb, tb, 0, h->stream>>>(P);
    else
        k_nt_fallback<0><<<(P.win_ncell + tb - 1) / tb, tb, 0, h->stream>>>(P);
}

// the Newton pipeline of one step (after k_columns)
static int launch_newton(Handle* h, Params& P, int* launches, bool timed, bool capturing) {
    int rc = newton_prepare(h, P);
    if (rc) return rc;
    const bool mixed = h->solver == REPROBUS_SOLVER_NEWTON_MIXED;
    if ((rc = enqueue_setup(h, P, mixed))) return rc;
    if ((rc = newton_solve(h, P, timed ? h->ev2 : nullptr, timed ? h->ev3 : nullptr, capturing))) return rc;
    if (h->mlp) {
        // the restart on its own stream while this one writes back the cells
        // that converged and then the fallback answers of the restart's cells
        const int tb = 128;
        if (!h->rstream) {
            int lo = 0, hi = 0;
            CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
            CUDA_TRY(cudaStreamCreateWithPriority(&h->rstream, cudaStreamNonBlocking, hi));
        }
        CUDA_TRY(cudaEventRecord(h->ev_fork, h->stream));
        k_nt_finish<0><<<(P.win_ncell + tb - 1) / tb, tb, 0, h->stream>>>(P);
        CUDA_TRY(cudaStreamWaitEvent(h->rstream, h->ev_fork, 0));
        if ((rc = newton_restart(h, P, h->rstream, h->stream, launches))) return rc;
        CUDA_TRY(cudaEventRecord(h->ev_join, h->rstream));
        CUDA_TRY(cudaStreamWaitEvent(h->stream, h->ev_join, 0));
        k_nt_fallback<1><<<(P.win_ncell + tb - 1) / tb, tb, 0, h->stream>>>(P);
    } else {
        newton_back(h, P);
    }
    *launches += mixed ? 6 : 5;  // setup, start (FP32 + FP64 redo), solve, finish, fallback
    return REPROBUS_OK;
}

// enqueue the kernels of one step on h->stream (device arrays in P)
// the work of one step on h->stream (device arrays in P); capturing: the
// calls are being recorded into a CUDA graph (events become graph nodes)
static int enqueue_step(Handle* h, Params& P, bool capturing, int* launches) {
    const int tb = 128;
    const bool counters = P.check || h->solver != REPROBUS_SOLVER_REF5;
    if (counters) CUDA_TRY(cudaMemsetAsync(h->d_count, 0, 8 * sizeof(unsigned long long), h->stream));
    k_columns<<<(P.ncol + tb - 1) / tb, tb, 0, h->stream>>>(P);
    (*launches)++;
    if (h->solver == REPROBUS_SOLVER_REF5 && !h->split_ref5) {
        k_chem<false, SETUP_TB, true><<<(unsigned)((P.ncell + SETUP_TB - 1) / SETUP_TB), SETUP_TB, 0, h->stream>>>(P);
        (*launches)++;
    } else if (h->solver == REPROBUS_SOLVER_REF5) {
        if (!capturing) {
            int rc = ensure_newton(h);
            if (rc) return rc;
        }
        P.nt_rec = h->nt_rec;
        launch_setup(h, P, false);
        k_ref_passes<<<(P.ncell + tb - 1) / tb, tb, 0, h->stream>>>(P);
        *launches += 2;
    } else {
        int rc = launch_newton(h, P, launches, true, capturing);
        if (rc) return rc;
    }
    if (P.fuse && h->nivbas < h->niv) {
        long long nt = (long long)P.nlon * P.nrows * (h->niv - h->nivbas);
        k_tail<<<(unsigned)((nt + 255) / 256), 256, 0, h->stream>>>(P);
        (*launches)++;
    }
    CUDA_TRY(cudaGetLastError());
    return REPROBUS_OK;
}

// Statistics of the step just enqueued on h->stream (ev0 recorded before it,
// ev2/ev3 around the solve), and the CHECK_FINITE verdict.
static int step_stats(Handle* h, const Params& P, reprobus_stats* st, int launches, bool graph) {
    const bool counters = P.check || h->solver != REPROBUS_SOLVER_REF5;
    if (st) {
        CUDA_TRY(cudaEventRecord(h->ev1, h->stream));
        CUDA_TRY(cudaEventSynchronize(h->ev1));
        float ms = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
        st->device_ms = ms;
        st->solve_ms = 0.;
        if (h->solver != REPROBUS_SOLVER_REF5) {
            float sm = 0.f;
            CUDA_TRY(cudaEventElapsedTime(&sm, h->ev2, h->ev3));
            st->solve_ms = sm;
        }
        st->ncells = P.ncell;
        st->kernel_launches = launches;
        st->passes = h->solver == REPROBUS_SOLVER_REF5 ? h->niter : h->npass;
        st->nonfinite = 0;
        st->newton_iters = 0;
        st->fallbacks = 0;
        st->max_newton_iters = 0;
        st->solver = h->solver;
        const int ip = h->solver == REPROBUS_SOLVER_NEWTON_MIXED ? 0 : 1;
        st->lanes_per_block = h->solver == REPROBUS_SOLVER_REF5 || !h->nt_var[ip] ? 0 : h->nt_var[ip]->nth;
        st->blocks_per_sm = h->solver == REPROBUS_SOLVER_REF5 ? 0 : h->nt_bps[ip];
        st->z_shared = h->solver == REPROBUS_SOLVER_REF5 || !h->nt_var[ip] ? 0 : h->nt_var[ip]->zshared;
        st->warm_start = h->solver != REPROBUS_SOLVER_REF5 && h->mlp ? 1 : 0;
        st->warm_restarts = 0;
        st->failed_iters = 0;
        st->start64_cells = 0;
        st->graph = graph ? 1 : 0;
    }
    if (counters && (st || P.check)) {
        unsigned long long c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        CUDA_TRY(cudaMemcpyAsync(c, h->d_count, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(cudaStreamSynchronize(h->stream));
        if (st) {
            st->nonfinite = (long long)c[0];
            st->newton_iters = (long long)c[1];
            st->fallbacks = (long long)c[2];
            st->max_newton_iters = (int)c[3];
            st->warm_restarts = (long long)c[4];
            st->failed_iters = (long long)c[5];
            st->start64_cells = (long long)c[6];
        }
        if (c[7])
            return set_err(REPROBUS_ERR_TIMEOUT,
                           "the learned restart's inference gave up waiting (its cells started again from the plain "
                           "start)");
        if (P.check && c[0]) return set_err(REPROBUS_ERR_NONFINITE, "%llu non-finite values in the step output", c[0]);
    }
    return REPROBUS_OK;
}

// which solver configuration a step runs (graphs are reused per configuration)
static int step_signature(const Handle* h) { return h->solver * 2 + (h->mlp ? 1 : 0); }

// One step: directly, or (REPROBUS_USE_GRAPH, once this configuration has run
// once directly, so that its buffers exist and its solve kernel is tuned) as
// a CUDA graph: the step's calls are captured, the handle's executable graph
// is updated in place (or instantiated), and launched as one unit.
static int launch_step(Handle* h, Params& P, reprobus_stats* st) {
    int launches = 0;
    P.fuse = (h->flags & REPROBUS_FUSE_CONSERV) ? 1 : 0;
    P.check = (h->flags & REPROBUS_CHECK_FINITE) ? 1 : 0;
    const int sig = step_signature(h);
    const bool graph = (h->flags & REPROBUS_USE_GRAPH) && (h->graph_ready & (1u << sig));
    if (st) CUDA_TRY(cudaEventRecord(h->ev0, h->stream));
    if (!graph) {
        int rc = enqueue_step(h, P, false, &launches);
        if (rc) return rc;
        h->graph_ready |= 1u << sig;
    } else {
        cudaGraph_t g = nullptr;
        CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue_step(h, P, true, &launches);
        const cudaError_t e = cudaStreamEndCapture(h->stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        CUDA_TRY(e);
        if (h->gexec && h->gexec_sig == sig) {
            cudaGraphExecUpdateResultInfo info;
            if (cudaGraphExecUpdate(h->gexec, g, &info) != cudaSuccess) {
                cudaGetLastError();
                cudaGraphExecDestroy(h->gexec);
                h->gexec = nullptr;
            }
        } else if (h->gexec) {
            cudaGraphExecDestroy(h->gexec);
            h->gexec = nullptr;
        }
        if (!h->gexec) {
            const cudaError_t ei = cudaGraphInstantiate(&h->gexec, g, 0);
            if (ei != cudaSuccess) {
                cudaGraphDestroy(g);
                h->gexec = nullptr;
                return set_err(REPROBUS_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(ei));
            }
            h->gexec_sig = sig;
        }
        cudaGraphDestroy(g);
        CUDA_TRY(cudaGraphLaunch(h->gexec, h->stream));
    }
    return step_stats(h, P, st, launches, graph);
}

extern "C" int reprobus_chem_set_tuning(void* handle, int lanes_per_block, int blocks_per_sm, int zshared) {
    Handle* h = (Handle*)handle;
    if (!h) return set_err(REPROBUS_ERR_ARG, "handle is NULL");
    if (lanes_per_block < 0 || blocks_per_sm < 0) return set_err(REPROBUS_ERR_ARG, "bad tuning values");
    if (zshared < 0 || zshared > 6) return set_err(REPROBUS_ERR_ARG, "zshared must be 0 .. 6");
    if (lanes_per_block > 0) {
        bool found = false;
        const NtVariant* vs[32];
        for (int m = 0; m < 2; m++) {
            const int nv = nt_all_variants(m == 0, vs, 32);
            for (int i = 0; i < nv; i++) found |= vs[i]->nth == lanes_per_block && vs[i]->zshared == zshared;
        }
        if (!found)
            return set_err(REPROBUS_ERR_ARG, "no solve-kernel shape with %d lanes per block (zshared %d)",
                           lanes_per_block, zshared);
    }
    h->want_lanes = lanes_per_block;
    h->want_zs = zshared;
    h->want_bps = blocks_per_sm;
    h->nt_var[0] = h->nt_var[1] = nullptr;
    h->nt_bps[0] = h->nt_bps[1] = 0;
    return REPROBUS_OK;
}

extern "C" int reprobus_chem_set_graph(void* handle, int on) {
    Handle* h = (Handle*)handle;
    if (!h) return set_err(REPROBUS_ERR_ARG, "handle is NULL");
    h->flags = on ? (h->flags | REPROBUS_USE_GRAPH) : (h->flags & ~REPROBUS_USE_GRAPH);
    return REPROBUS_OK;
}

extern "C" int reprobus_chem_set_mlp(void* handle, void* net) {
    Handle* h = (Handle*)handle;
    if (!h) return set_err(REPROBUS_ERR_ARG, "handle is NULL");
    if (h->mlp != net) h->graph_ready &= ~(1u << (h->solver * 2 + 1));  // a new network runs directly once
    h->mlp = net;
    return REPROBUS_OK;
}

__global__ void __launch_bounds__(128) k_features(Params P) {
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= P.ncell) return;
    CellPro C;
    cell_prologue<true>(P, cell, C);
    double ck[NBCON], cc[NCM];
#pragma unroll
    for (int n = 0; n < NBCON; n++) ck[n] = C.ck0[n];
#pragma unroll
    for (int n = 0; n < NCM; n++) cc[n] = C.cc0[n];
#pragma unroll 1
    for (int it = 0; it < P.npass; it++) cell_pass(C.F, C.K, C.tj, C.A.het, C.ck0, P.sc.dt, ck, cc);
    float fe[64];
    cell_features(P, C.g, C.F.hnm, C.F.sza, C.A.surf, ck, cc, fe);
    float4* o = reinterpret_cast<float4*>(P.mlp_feat + (size_t)cell * 64);
#pragma unroll
    for (int i = 0; i < 16; i++) o[i] = make_float4(fe[4 * i], fe[4 * i + 1], fe[4 * i + 2], fe[4 * i + 3]);
}

extern "C" int reprobus_chem_features_dev(void* handle, int ilat0, int ilat1, double daynum, double dt,
                                          const double* alt,
                                          const double* trajlon, const double* trajlat, const double* trajpre,
                                          const double* trajtem, int irapp, const double* qj1, const double* hc,
                                          float* feat) {
    Handle* h = (Handle*)handle;
    if (!h) return set_err(REPROBUS_ERR_ARG, "handle is NULL");
    int rc = check_rows(h, ilat0, ilat1);
    if (rc) return rc;
    if (irapp < 1 || irapp > h->nrappmax) return set_err(REPROBUS_ERR_ARG, "irapp %d outside 1..%d", irapp, h->nrappmax);
    if (!alt || !trajlon || !trajlat || !trajpre || !trajtem || !qj1 || !hc || !feat)
        return set_err(REPROBUS_ERR_ARG, "NULL array argument");
    if (((uintptr_t)feat) & 15) return set_err(REPROBUS_ERR_ARG, "feat must be 16-byte aligned");
    Params P;
    fill_params(h, P, ilat0, ilat1);
    P.trajoff = (long long)(irapp - 1) * h->nlon * h->nlat * h->niv;
    P.alt = alt;
    P.trajlon = trajlon;
    P.trajlat = trajlat;
    P.trajpre = trajpre;
    P.trajtem = trajtem;
    P.qj1 = const_cast<double*>(qj1);  // read only (DIAG prologue)
    P.hc = const_cast<double*>(hc);
    P.mlp_feat = feat;
    step_const(h, daynum, dt, P.sc);
    const int tb = 128;
    k_columns<<<(P.ncol + tb - 1) / tb, tb, 0, h->stream>>>(P);
    k_features<<<(P.ncell + tb - 1) / tb, tb, 0, h->stream>>>(P);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return REPROBUS_OK;
}

extern "C" int reprobus_chem_set_solver(void* handle, int solver, int npass, int maxit, double tol) {
    Handle* h = (Handle*)handle;
    if (!h) return set_err(REPROBUS_ERR_ARG, "handle is NULL");
    if (solver < REPROBUS_SOLVER_REF5 || solver > REPROBUS_SOLVER_NEWTON_MIXED)
        return set_err(REPROBUS_ERR_ARG, "unknown solver %d", solver);
    if (npass < 0 || maxit < 1 || !(tol > 0.)) return set_err(REPROBUS_ERR_ARG, "bad npass/maxit/tol");
    h->solver = solver;
    h->npass = npass;
    h->maxit = maxit;
    h->tol = tol;
    return REPROBUS_OK;
}

extern "C" int reprobus_chem_step_dev(void* handle, int ilat0, int ilat1, double daynum, double dt, const double* alt,
                                      const double* trajlon, const double* trajlat, const double* trajpre,
                                      const double* trajtem, int irapp, double* qj1, double* hc, double* vsed3d,
                                      double* parth2osed, double* parthno3sed, double* surfarea, double* sza3d,
                                      reprobus_stats* stats) {
    Handle* h = (Handle*)handle;
    if (!h) return set_err(REPROBUS_ERR_ARG, "handle is NULL");
    int rc = check_rows(h, ilat0, ilat1);
    if (rc) return rc;
    if (irapp < 1 || irapp > h->nrappmax) return set_err(REPROBUS_ERR_ARG, "irapp %d outside 1..%d", irapp, h->nrappmax);
    if (!alt || !trajlon || !trajlat || !trajpre || !trajtem || !qj1 || !hc || !vsed3d || !parth2osed ||
        !parthno3sed || !surfarea || !sza3d)
        return set_err(REPROBUS_ERR_ARG, "NULL array argument");
    Params P;
    fill_params(h, P, ilat0, ilat1);
    P.trajoff = (long long)(irapp - 1) * h->nlon * h->nlat * h->niv;
    P.alt = alt;
    P.trajlon = trajlon;
    P.trajlat = trajlat;
    P.trajpre = trajpre;
    P.trajtem = trajtem;
    P.qj1 = qj1;
    P.hc = hc;
    P.vsed3d = vsed3d;
    P.parth2osed = parth2osed;
    P.parthno3sed = parthno3sed;
    P.surfarea = surfarea;
    P.sza3d = sza3d;
    step_const(h, daynum, dt, P.sc);
    return launch_step(h, P, stats);
}

// strided copy of rows [r0, r0+nr) of `planes` consecutive (nlon,nlat) planes;
// all rows of the planes are one contiguous range: one linear copy (the 2-D
// copy path moves whole planes markedly slower)
static int copy_rows(double* dst, const double* src, const Handle* h, int r0, int nr, size_t plane0, size_t planes,
                     cudaMemcpyKind kind, cudaStream_t s) {
    const size_t pitch = (size_t)h->nlon * h->nlat * sizeof(double);
    const size_t off = plane0 * h->nlon * h->nlat + (size_t)h->nlon * r0;
    if (nr == h->nlat) {
        CUDA_TRY(cudaMemcpyAsync(dst + off, src + off, pitch * planes, kind, s));
        return REPROBUS_OK;
    }
    CUDA_TRY(cudaMemcpy2DAsync(dst + off, pitch, src + off, pitch, (size_t)h->nlon * nr * sizeof(double), planes,
                               kind, s));
    return REPROBUS_OK;
}

constexpr int HOST_CHUNK_MIN_ROWS = 8;  // rows per chunk of the host-array entry point at least

static int ensure_mirrors(Handle* h) {
    if (h->m_qj1) return REPROBUS_OK;
    const size_t pl = (size_t)h->nlon * h->nlat * h->niv;
    const size_t pb = (size_t)h->nlon * h->nlat * h->nivbas;
    CUDA_TRY(cudaMalloc(&h->m_alt, pl * sizeof(double)));
    for (auto& p : h->m_traj) CUDA_TRY(cudaMalloc(&p, pl * sizeof(double)));
    CUDA_TRY(cudaMalloc(&h->m_qj1, pl * NBCON * sizeof(double)));
    CUDA_TRY(cudaMalloc(&h->m_hc, pl * NCM * sizeof(double)));
    for (int q = 0; q < 4; q++) CUDA_TRY(cudaMalloc(&h->m_out[q], pb * sizeof(double)));
    CUDA_TRY(cudaMalloc(&h->m_out[4], pl * sizeof(double)));
    return REPROBUS_OK;
}

// the host arrays of rows [r0, r0 + nr) into the handle's device mirrors
// (alt and the irapp slice of traj* on levels 1..nivbas, the state) or back
// (state and diagnostics), on stream s
struct HostArrays {
    const double* alt;
    const double* traj[4];
    double *qj1, *hc, *vsed3d, *parth2osed, *parthno3sed, *surfarea, *sza3d;
};

static int host_rows_in(Handle* h, const HostArrays& A, int r0, int nr, cudaStream_t s) {
    const size_t nb = h->nivbas, niv = h->niv;
    const bool fuse = (h->flags & REPROBUS_FUSE_CONSERV) != 0;
    const cudaMemcpyKind H2D = cudaMemcpyHostToDevice;
    int rc;
    if ((rc = copy_rows(h->m_alt, A.alt, h, r0, nr, 0, nb, H2D, s))) return rc;
    for (int q = 0; q < 4; q++)
        if ((rc = copy_rows(h->m_traj[q], A.traj[q], h, r0, nr, 0, nb, H2D, s))) return rc;
    if (fuse || nb == niv) {
        if ((rc = copy_rows(h->m_qj1, A.qj1, h, r0, nr, 0, niv * NBCON, H2D, s))) return rc;
    } else {
        for (int n = 0; n < NBCON; n++)
            if ((rc = copy_rows(h->m_qj1, A.qj1, h, r0, nr, niv * n, nb, H2D, s))) return rc;
    }
    for (int n = 0; n < NCM; n++)
        if ((rc = copy_rows(h->m_hc, A.hc, h, r0, nr, niv * n, nb, H2D, s))) return rc;
    return REPROBUS_OK;
}

static int host_rows_out(Handle* h, const HostArrays& A, int r0, int nr, cudaStream_t s) {
    const size_t nb = h->nivbas, niv = h->niv;
    const bool fuse = (h->flags & REPROBUS_FUSE_CONSERV) != 0;
    const cudaMemcpyKind D2H = cudaMemcpyDeviceToHost;
    int rc;
    if (fuse || nb == niv) {
        if ((rc = copy_rows(A.qj1, h->m_qj1, h, r0, nr, 0, niv * NBCON, D2H, s))) return rc;
    } else {
        for (int n = 0; n < NBCON; n++)
            if ((rc = copy_rows(A.qj1, h->m_qj1, h, r0, nr, niv * n, nb, D2H, s))) return rc;
    }
    for (int n = 0; n < NCM; n++)
        if ((rc = copy_rows(A.hc, h->m_hc, h, r0, nr, niv * n, nb, D2H, s))) return rc;
    if ((rc = copy_rows(A.vsed3d, h->m_out[0], h, r0, nr, 0, nb, D2H, s))) return rc;
    if ((rc = copy_rows(A.parth2osed, h->m_out[1], h, r0, nr, 0, nb, D2H, s))) return rc;
    if ((rc = copy_rows(A.parthno3sed, h->m_out[2], h, r0, nr, 0, nb, D2H, s))) return rc;
    if ((rc = copy_rows(A.sza3d, h->m_out[3], h, r0, nr, 0, nb, D2H, s))) return rc;
    const size_t kh = h->nivhau - 1;
    if ((rc = copy_rows(A.surfarea, h->m_out[4], h, r0, nr, kh, nb - kh, D2H, s))) return rc;
    return REPROBUS_OK;
}

static void add_stats(reprobus_stats* acc, const reprobus_stats& c, bool first) {
    if (first) {
        *acc = c;
        return;
    }
    acc->ncells += c.ncells;
    acc->nonfinite += c.nonfinite;
    acc->kernel_launches += c.kernel_launches;
    acc->device_ms += c.device_ms;
    acc->newton_iters += c.newton_iters;
    acc->fallbacks += c.fallbacks;
    if (c.max_newton_iters > acc->max_newton_iters) acc->max_newton_iters = c.max_newton_iters;
    acc->warm_restarts += c.warm_restarts;
    acc->failed_iters += c.failed_iters;
    acc->solve_ms += c.solve_ms;
    acc->start64_cells += c.start64_cells;
}

// P over rows a..b (1-based) of the handle's device mirrors of the host arrays
static void mirror_params(Handle* h, Params& P, int a, int b, double daynum, double dt) {
    fill_params(h, P, a, b);
    P.trajoff = 0;
    P.alt = h->m_alt;
    P.trajlon = h->m_traj[0];
    P.trajlat = h->m_traj[1];
    P.trajpre = h->m_traj[2];
    P.trajtem = h->m_traj[3];
    P.qj1 = h->m_qj1;
    P.hc = h->m_hc;
    P.vsed3d = h->m_out[0];
    P.parth2osed = h->m_out[1];
    P.parthno3sed = h->m_out[2];
    P.sza3d = h->m_out[3];
    P.surfarea = h->m_out[4];
    step_const(h, daynum, dt, P.sc);
}

// rows r0..r0+nr-1 of P's range as the window of the per-cell kernels
static void set_window(Params& P, int r0, int nr) {
    P.win_r0 = r0;
    P.win_nr = nr;
    P.win_ncol = P.nlon * nr;
    P.win_ncell = P.win_ncol * P.nivbas;
}

// A Newton step through the host arrays in row chunks. The rate stage and
// plain start of chunk c run as soon as its rows are in (stream cin). The
// cells of chunks 0 .. nchunk-2 and those of the last chunk then form two
// work queues, solved one after the other by the persistent kernel; the
// write-back of the first chunks runs between the two solves and their
// copies out (stream cout) during the second, so that only the last chunk's
// write-back and copy out follow it. Chunk c holds rows ilat0 + nrows c / nchunk ..
// ilat0 + nrows (c + 1) / nchunk - 1.
static int host_step_newton(Handle* h, const HostArrays& A, int ilat0, int ilat1, int nchunk, double daynum,
                            double dt, reprobus_stats* st) {
    const bool mixed = h->solver == REPROBUS_SOLVER_NEWTON_MIXED;
    const int nrows = ilat1 - ilat0 + 1, tb = 128;
    Params P;
    mirror_params(h, P, ilat0, ilat1, daynum, dt);
    P.fuse = (h->flags & REPROBUS_FUSE_CONSERV) ? 1 : 0;
    P.check = (h->flags & REPROBUS_CHECK_FINITE) ? 1 : 0;
    int rc = newton_prepare(h, P);
    if (rc) return rc;
    auto row0 = [&](int c) { return ilat0 + (int)((long long)nrows * c / nchunk); };
    // queue of the first chunks (heads nt_head[0..2]) and of the last (nt_head[4..6])
    Params PA = P, PB = P;
    PA.nt_qcap = P.nlon * (row0(nchunk - 1) - ilat0) * P.nivbas;
    PB.nt_qcap = P.ncell - PA.nt_qcap;
    PB.nt_list = P.nt_list + PA.nt_qcap;
    PB.nt_head = P.nt_head + 4;
    const bool tail = P.fuse && h->nivbas < h->niv;
    int launches = 0;
    if (st) CUDA_TRY(cudaEventRecord(h->ev0, h->stream));
    CUDA_TRY(cudaMemsetAsync(h->d_count, 0, 8 * sizeof(unsigned long long), h->stream));
    CUDA_TRY(cudaMemsetAsync(h->nt_head, 0, 8 * sizeof(int), h->stream));
    for (int c = 0; c < nchunk; c++) {
        const int a = row0(c), b = row0(c + 1) - 1;
        if ((rc = host_rows_in(h, A, a - 1, b - a + 1, h->cin))) return rc;
        CUDA_TRY(cudaEventRecord(h->ev_in[c], h->cin));
        CUDA_TRY(cudaStreamWaitEvent(h->stream, h->ev_in[c], 0));
        Params& Q = c < nchunk - 1 ? PA : PB;
        set_window(Q, a - ilat0, b - a + 1);
        k_columns<<<(Q.win_ncol + tb - 1) / tb, tb, 0, h->stream>>>(Q);
        newton_front(h, Q, mixed);
        launches += mixed ? 4 : 3;
    }
    set_window(P, 0, nrows);
    for (int part = 0; part < 2; part++) {
        Params& Q = part == 0 ? PA : PB;
        if ((rc = newton_solve(h, Q, st ? (part ? h->ev4 : h->ev2) : nullptr, st ? (part ? h->ev5 : h->ev3) : nullptr,
                               false)))
            return rc;
        launches++;
        if (h->mlp) {  // over the rows of this queue
            const int a = part == 0 ? row0(0) : row0(nchunk - 1), b = part == 0 ? row0(nchunk - 1) : ilat1 + 1;
            set_window(Q, a - ilat0, b - a);
            if ((rc = newton_restart(h, Q, h->stream, h->stream, &launches))) return rc;
        }
        for (int c = part == 0 ? 0 : nchunk - 1; c < (part == 0 ? nchunk - 1 : nchunk); c++) {
            const int a = row0(c), b = row0(c + 1) - 1;
            set_window(Q, a - ilat0, b - a + 1);
            newton_back(h, Q);
            launches += 2;
            if (tail) {
                const long long nt = (long long)Q.nlon * Q.win_nr * (h->niv - h->nivbas);
                k_tail<<<(unsigned)((nt + 255) / 256), 256, 0, h->stream>>>(Q);
                launches++;
            }
            CUDA_TRY(cudaGetLastError());
            CUDA_TRY(cudaEventRecord(h->ev_comp[c], h->stream));
            CUDA_TRY(cudaStreamWaitEvent(h->cout, h->ev_comp[c], 0));
            if ((rc = host_rows_out(h, A, a - 1, b - a + 1, h->cout))) return rc;
        }
    }
    rc = step_stats(h, P, st, launches, false);
    if (!rc && st) {  // the two solves
        float sb = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&sb, h->ev4, h->ev5));
        st->solve_ms += sb;
    }
    return rc;
}

extern "C" int reprobus_chem_step(void* handle, int ilat0, int ilat1, double daynum, double dt, const double* alt,
                                  const double* trajlon, const double* trajlat, const double* trajpre,
                                  const double* trajtem, int irapp, double* qj1, double* hc, double* vsed3d,
                                  double* parth2osed, double* parthno3sed, double* surfarea, double* sza3d,
                                  reprobus_stats* stats) {
    Handle* h = (Handle*)handle;
    if (!h) return set_err(REPROBUS_ERR_ARG, "handle is NULL");
    int rc = check_rows(h, ilat0, ilat1);
    if (rc) return rc;
    if (irapp < 1 || irapp > h->nrappmax) return set_err(REPROBUS_ERR_ARG, "irapp %d outside 1..%d", irapp, h->nrappmax);
    if (!alt || !trajlon || !trajlat || !trajpre || !trajtem || !qj1 || !hc || !vsed3d || !parth2osed ||
        !parthno3sed || !surfarea || !sza3d)
        return set_err(REPROBUS_ERR_ARG, "NULL array argument");
    if ((rc = ensure_mirrors(h))) return rc;
    const size_t pl = (size_t)h->nlon * h->nlat * h->niv;
    const HostArrays A{alt,
                       {trajlon + (irapp - 1) * pl, trajlat + (irapp - 1) * pl, trajpre + (irapp - 1) * pl,
                        trajtem + (irapp - 1) * pl},
                       qj1, hc, vsed3d, parth2osed, parthno3sed, surfarea, sza3d};
    // Rows in chunks (4, or REPROBUS_HOST_CHUNKS): the copy of chunk c+1 in
    // (stream cin) and of chunk c-1 out (stream cout) run while chunk c
    // integrates on the handle's stream; chunks touch disjoint rows of the
    // device mirrors, and the order is carried by events (no kernel waits on
    // another). REF5, the first Newton step (its autotuning) and graph
    // launches integrate chunk by chunk (statistics and CHECK_FINITE
    // synchronise per chunk); a tuned Newton step runs in phases instead
    // (host_step_newton).
    const int nrows = ilat1 - ilat0 + 1;
    int want_chunks = 4;
    if (const char* ev = getenv("REPROBUS_HOST_CHUNKS")) {
        const int v = atoi(ev);
        if (v >= 1 && v <= 4) want_chunks = v;
    }
    int nchunk = want_chunks;
    while (nchunk > 1 && nrows < nchunk * HOST_CHUNK_MIN_ROWS) nchunk--;
    if (nchunk > 1 && !h->cin) {
        CUDA_TRY(cudaStreamCreateWithFlags(&h->cin, cudaStreamNonBlocking));
        CUDA_TRY(cudaStreamCreateWithFlags(&h->cout, cudaStreamNonBlocking));
        for (int c = 0; c < 4; c++) {
            CUDA_TRY(cudaEventCreateWithFlags(&h->ev_in[c], cudaEventDisableTiming));
            CUDA_TRY(cudaEventCreateWithFlags(&h->ev_comp[c], cudaEventDisableTiming));
        }
    }
    cudaStream_t cin = nchunk > 1 ? h->cin : h->stream, cout = nchunk > 1 ? h->cout : h->stream;
    if (nchunk > 1) {  // the copies in must not overtake work still queued on the handle's stream
        CUDA_TRY(cudaEventRecord(h->ev_comp[3], h->stream));
        CUDA_TRY(cudaStreamWaitEvent(cin, h->ev_comp[3], 0));
    }
    reprobus_stats acc, one;
    // on an error, let the copies already queued finish before returning
    auto fail = [&](int code) {
        cudaStreamSynchronize(cin);
        cudaStreamSynchronize(cout);
        return code;
    };
    // Newton solvers, once their solve kernel is tuned (the tuning times
    // candidates on cells already on the device) and without a graph: one
    // solve over all chunks
    const int ip = h->solver == REPROBUS_SOLVER_NEWTON_MIXED ? 0 : 1;
    if (nchunk > 1 && h->solver != REPROBUS_SOLVER_REF5 && !(h->flags & REPROBUS_USE_GRAPH) && h->nt_var[ip]) {
        if ((rc = host_step_newton(h, A, ilat0, ilat1, nchunk, daynum, dt, stats))) return fail(rc);
        CUDA_TRY(cudaStreamSynchronize(cout));
        return REPROBUS_OK;
    }
    for (int c = 0; c < nchunk; c++) {
        const int a = ilat0 + (int)((long long)nrows * c / nchunk);
        const int b = ilat0 + (int)((long long)nrows * (c + 1) / nchunk) - 1;
        if ((rc = host_rows_in(h, A, a - 1, b - a + 1, cin))) return fail(rc);
        if (nchunk > 1) {
            CUDA_TRY(cudaEventRecord(h->ev_in[c], cin));
            CUDA_TRY(cudaStreamWaitEvent(h->stream, h->ev_in[c], 0));
        }
        Params P;
        mirror_params(h, P, a, b, daynum, dt);
        if ((rc = launch_step(h, P, stats ? &one : nullptr))) return fail(rc);
        if (stats) add_stats(&acc, one, c == 0);
        if (nchunk > 1) {
            CUDA_TRY(cudaEventRecord(h->ev_comp[c], h->stream));
            CUDA_TRY(cudaStreamWaitEvent(cout, h->ev_comp[c], 0));
        }
        if ((rc = host_rows_out(h, A, a - 1, b - a + 1, cout))) return fail(rc);
    }
    CUDA_TRY(cudaStreamSynchronize(cout));
    if (stats) *stats = acc;
    return REPROBUS_OK;
}

extern "C" int reprobus_chem_rates_dev(void* handle, int ilat0, int ilat1, double daynum, const double* alt,
                                       const double* trajlon, const double* trajlat, const double* trajpre,
                                       const double* trajtem, int irapp, const double* qj1, const double* hc,
                                       double* diag) {
    Handle* h = (Handle*)handle;
    if (!h) return set_err(REPROBUS_ERR_ARG, "handle is NULL");
    int rc = check_rows(h, ilat0, ilat1);
    if (rc) return rc;
    if (irapp < 1 || irapp > h->nrappmax) return set_err(REPROBUS_ERR_ARG, "irapp %d outside 1..%d", irapp, h->nrappmax);
    if (!alt || !trajlon || !trajlat || !trajpre || !trajtem || !qj1 || !hc || !diag)
        return set_err(REPROBUS_ERR_ARG, "NULL array argument");
    Params P;
    fill_params(h, P, ilat0, ilat1);
    P.trajoff = (long long)(irapp - 1) * h->nlon * h->nlat * h->niv;
    P.alt = alt;
    P.trajlon = trajlon;
    P.trajlat = trajlat;
    P.trajpre = trajpre;
    P.trajtem = trajtem;
    P.qj1 = const_cast<double*>(qj1);  // read only in the DIAG instantiation
    P.hc = const_cast<double*>(hc);
    P.diag = diag;
    step_const(h, daynum, 0., P.sc);
    const int tb = 128;
    k_columns<<<(P.ncol + tb - 1) / tb, tb, 0, h->stream>>>(P);
    k_chem<true><<<(P.ncell + tb - 1) / tb, tb, 0, h->stream>>>(P);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return REPROBUS_OK;
}

extern "C" int reprobus_conserv_dev(void* handle, int ilat0, int ilat1, double* qj1, double* hc) {
    Handle* h = (Handle*)handle;
    if (!h) return set_err(REPROBUS_ERR_ARG, "handle is NULL");
    int rc = check_rows(h, ilat0, ilat1);
    if (rc) return rc;
    if (!qj1 || !hc) return set_err(REPROBUS_ERR_ARG, "NULL array argument");
    Params P;
    fill_params(h, P, ilat0, ilat1);
    P.qj1 = qj1;
    P.hc = hc;
    long long n = (long long)h->nlon * P.nrows * h->niv;
    k_conserv<<<(unsigned)((n + 127) / 128), 128, 0, h->stream>>>(P);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return REPROBUS_OK;
}

// ----------------------------------------------------------------------------
// Allocation-free step (no counterpart in the reference).
//
// Some callers may not allocate device memory once they are running: a model
// whose GPU memory is reserved up front and handed out by its own runtime or
// pool (an OpenACC/CUDA-Fortran data region, a framework's caching
// allocator), or a process held to a fixed device-memory budget. For them,
// reprobus_chem_step_noalloc takes every array from the caller and keeps the
// only scratch the step needs (the column sums written by k_columns and read
// by k_chem, and the non-finite counter) in the fixed array below, which the
// CUDA runtime places on each device when the library's module is loaded
// there and keeps until the process exits. The kernels and their launch are
// those of reprobus_chem_step_dev.
// ----------------------------------------------------------------------------
#include <mutex>

static __device__ __align__(256) double g_noalloc_scratch[REPROBUS_NOALLOC_SCRATCH_DOUBLES];

// In host code g_noalloc_scratch names a host-side stand-in, not device
// memory: its device address is looked up once per device (with that device
// current) and cached here. A cached address is confirmed on each call by a
// pointer-attribute query (host-side, no allocation); after cudaDeviceReset
// the module is loaded again in a new context, the old address no longer
// belongs to the device, and it is looked up again.
static std::mutex g_noalloc_mu;
static double* g_noalloc_dev[256];

static int noalloc_scratch(double** out) {
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) return set_err(REPROBUS_ERR_ARG, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (g_noalloc_dev[dev]) {
        cudaPointerAttributes pa;
        if (cudaPointerGetAttributes(&pa, g_noalloc_dev[dev]) != cudaSuccess || pa.type != cudaMemoryTypeDevice ||
            pa.device != dev) {
            cudaGetLastError();  // clear the error state the query may have left
            g_noalloc_dev[dev] = nullptr;
        }
    }
    if (!g_noalloc_dev[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return set_err(REPROBUS_ERR_CUDA, "cudaGetSymbolAddress(scratch) on device %d: %s", dev,
                           cudaGetErrorString(e));
        g_noalloc_dev[dev] = (double*)p;
    }
    *out = g_noalloc_dev[dev];
    return REPROBUS_OK;
}

extern "C" int reprobus_chem_step_noalloc(const double* ajl, const double* o3up, const double* troe, int nlon,
                                          int nlat, int niv, int nivbas, int nivhau, int nrappmax, int niter,
                                          int flags, int ilat0, int ilat1, double daynum, double dt,
                                          const double* alt, const double* trajlon, const double* trajlat,
                                          const double* trajpre, const double* trajtem, int irapp, double* qj1,
                                          double* hc, double* vsed3d, double* parth2osed, double* parthno3sed,
                                          double* surfarea, double* sza3d, void* stream) {
    if (!ajl || !o3up || !troe) return set_err(REPROBUS_ERR_ARG, "ajl, o3up and troe must be non-NULL");
    if (int rc = check_troe(troe)) return rc;
    if (nlon <= 0 || nlat <= 0 || niv <= 0 || nivbas <= 0 || nivbas > niv || nivhau < 1 || nivhau > nivbas ||
        nrappmax <= 0 || niter < 0)
        return set_err(REPROBUS_ERR_ARG, "bad sizes: nlon=%d nlat=%d niv=%d nivbas=%d nivhau=%d nrappmax=%d niter=%d",
                       nlon, nlat, niv, nivbas, nivhau, nrappmax, niter);
    if (ilat0 < 1 || ilat1 > nlat || ilat0 > ilat1)
        return set_err(REPROBUS_ERR_ARG, "bad row range %d..%d (nlat=%d)", ilat0, ilat1, nlat);
    if (irapp < 1 || irapp > nrappmax) return set_err(REPROBUS_ERR_ARG, "irapp %d outside 1..%d", irapp, nrappmax);
    if (!alt || !trajlon || !trajlat || !trajpre || !trajtem || !qj1 || !hc || !vsed3d || !parth2osed ||
        !parthno3sed || !surfarea || !sza3d)
        return set_err(REPROBUS_ERR_ARG, "NULL array argument");
    // scratch layout: [counter, padded to 256 B][3 doubles per cell][1 double per column]
    const long long nrows = ilat1 - ilat0 + 1;
    const long long ncol = (long long)nlon * nrows;
    const long long need = 32 + 3 * ncol * nivbas + ncol;
    if (need > REPROBUS_NOALLOC_SCRATCH_DOUBLES)
        return set_err(REPROBUS_ERR_ARG,
                       "rows %d..%d need %lld scratch doubles; the allocation-free step holds at most %d "
                       "(3*nlon*rows*nivbas + nlon*rows + 32): pass fewer rows per call",
                       ilat0, ilat1, need, REPROBUS_NOALLOC_SCRATCH_DOUBLES);
    double* scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    // a handle on the stack that owns nothing: the caller's table and the fixed scratch
    Handle h;
    h.nlon = nlon;
    h.nlat = nlat;
    h.niv = niv;
    h.nivbas = nivbas;
    h.nivhau = nivhau;
    h.nrappmax = nrappmax;
    h.niter = niter;
    h.flags = flags;
    CUDA_TRY(cudaGetDevice(&h.device));
    memcpy(h.troe, troe, sizeof(h.troe));
    h.d_ajl = const_cast<double*>(ajl);
    h.d_o3up = const_cast<double*>(o3up);
    h.d_count = reinterpret_cast<unsigned long long*>(scratch);
    h.d_col = scratch + 32;
    h.stream = (cudaStream_t)stream;
    h.split_ref5 = false;  // no record buffers: the single-kernel REF5
    Params P;
    fill_params(&h, P, ilat0, ilat1);
    P.trajoff = (long long)(irapp - 1) * nlon * nlat * niv;
    P.alt = alt;
    P.trajlon = trajlon;
    P.trajlat = trajlat;
    P.trajpre = trajpre;
    P.trajtem = trajtem;
    P.qj1 = qj1;
    P.hc = hc;
    P.vsed3d = vsed3d;
    P.parth2osed = parth2osed;
    P.parthno3sed = parthno3sed;
    P.surfarea = surfarea;
    P.sza3d = sza3d;
    step_const(&h, daynum, dt, P.sc);
    return launch_step(&h, P, nullptr);
}
