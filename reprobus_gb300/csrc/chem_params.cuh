// chem_params.cuh — launch parameters shared by the step kernels
// (chem_kernels.cu) and the Newton solve kernels (nt_solve_*.cu).
#pragma once
#include <cuda_runtime.h>

#include "chem_cell.cuh"

namespace rpb {

// ----------------------------------------------------------------------------
// kernel parameters
// ----------------------------------------------------------------------------
struct Params {
    int nlon, nlat, niv, nivbas, nivhau;
    int ilat0, nrows;          // 0-based first row, number of rows
    long long trajoff;         // element offset of the irapp slice in traj*
    int niter, fuse, check;
    int ncell, ncol;           // nlon*nrows*nivbas, nlon*nrows
    int win_r0, win_nr;        // row window of the per-cell kernels (rows of the range)
    int win_ncell, win_ncol;   // nlon*win_nr*nivbas, nlon*win_nr
    int nt_qcap;               // entries of the work queue nt_list (day from the front, night from the back)
    const double* __restrict__ alt;
    const double* __restrict__ trajlon;
    const double* __restrict__ trajlat;
    const double* __restrict__ trajpre;
    const double* __restrict__ trajtem;
    double* qj1;
    double* hc;
    double* vsed3d;
    double* parth2osed;
    double* parthno3sed;
    double* surfarea;
    double* sza3d;
    const double* __restrict__ ajl;
    const double* __restrict__ o3up;
    double* col;               // scratch: o3t | colo2 | colno (ncell each) | sza_top (ncol)
    unsigned long long* nonfinite;  // [0] non-finite values, [1] Newton iterations,
                                    // [2] fallbacks, [3] max iterations of a cell,
                                    // [4] cells restarted from the network's start,
                                    // [5] iterations of attempts that missed,
                                    // [6] FP64 redos of the FP32 start,
                                    // [7] the learned restart's inference timed out
    double* diag;
    int npass, maxit;               // Newton: reference passes before, iteration cap
    double tol;                     // Newton: scaled step tolerance
    // Newton state, one record per cell of the call (cell-major)
    double* nt_rec;                 // NT_REC FP64 fields: rates, fixed constants, day flag, ck0
    float* nt_rec32;                // NT_REC32 FP32 copies of the rate fields (mixed solver)
    double* nt_x;                   // iterate x (NT_NX per cell)
    int* nt_stat;                   // 0 active, >0 converged at that iteration (plus stat_bias), -1 failed
    int stat_bias;                  // added to the iterations of a converged cell: 0 for the solve from the
                                    // plain start, NT_RESTART_BIAS for the learned restart's solve
    int* nt_list;                   // work queue: day cells from the front, night cells from the back
    int* nt_head;                   // [0] next queue entry, [1] day count, [2] night count,
                                    // [3] cells taken for the learned restart
    int npass_plain;                // reference passes of the plain start
    // learned restart: a cell whose plain start misses the convergence test
    // gets slot k < mlp_cap; its features, the network's prediction and its
    // cell index are stored at slot k
    int mlp_cap;
    float* mlp_feat;                // 64 raw features per slot (row-major)
    const float* mlp_y;             // 64 predicted log10 end-of-step ratios per slot (57 used)
    int* mlp_cells;                 // the cell of each slot
    const unsigned int* mlp_err;    // the inference kernel's error flag: set, the predictions are not used
    StepConst sc;
};

// fields of a Newton cell record: K (99), tj (41), het (9), fixed constants
// (14: o2 n2 h2 co2 hnm parthno3 parth2o parthcl parthbr rain_hno3 rain_hcl
// rain_hbr rain_h2o2 dt), solar zenith angle (a cell is a day cell when it is
// <= 95 deg), start-of-step number densities ck0 (43), aerosol surface area
constexpr int NT_RK = 0, NT_RJ = NRATE, NT_RH = NRATE + NPHOT, NT_RF = NRATE + NPHOT + 9;
constexpr int NT_RSZA = NT_RF + 14, NT_RCK0 = NT_RSZA + 1, NT_RSURF = NT_RCK0 + NBCON;
constexpr int NT_REC = 208;    // FP64 record stride (1664 B = 13 lines of 128 B)
constexpr int NT_REC32 = 168;  // FP32 record stride (164 used)
constexpr int NT_RESTART_BIAS = 1 << 16;  // Params::stat_bias of the learned restart's solve
constexpr int NT_STAT_NOSLOT = -4;         // a cell that missed and found no slot of the restart
static_assert(NT_RSURF < NT_REC, "record layout");

__device__ __forceinline__ size_t plane3(const Params& P) { return (size_t)P.nlon * P.nlat * P.niv; }
__device__ __forceinline__ size_t plane_b(const Params& P) { return (size_t)P.nlon * P.nlat * P.nivbas; }


__device__ __forceinline__ size_t cell_global(const Params& P, int cell) {
    const int i = cell % P.nlon;
    const int rest = cell / P.nlon;
    const int k = rest / P.nrows;
    const int j = P.ilat0 + rest % P.nrows;
    return (size_t)i + (size_t)P.nlon * ((size_t)j + (size_t)P.nlat * k);
}

}  // namespace rpb
