// newton_kernel.cuh — the persistent Newton solve kernel of one step.
//
// One lane integrates one cell at a time. The lanes of a warp take cells from
// a global work queue (one atomic per warp and refill, lanes ranked by
// ballot): a lane whose cell has converged, failed or hit the iteration cap
// takes the next queue entry at the top of the loop, so cells needing 2 or 15
// iterations share a warp without idling it. The queue holds the day cells
// first and the night cells after them, so the lanes of a warp mostly run the
// same (day or night) equations.
//
// Per iteration (newton_solve.cuh): scaled Jacobian in TJ into the lane's
// NT_NSLOT shared-memory slots (slot-major, stride NTH: every slot access of
// a warp is one conflict-free row of banks), FP64 residual, Crout
// factorisation with fused forward substitution and back substitution in TJ,
// FP64 update of the iterate in the cell's record. ZS: the right-hand side
// and step z in NT_NX more shared-memory slots per lane (else registers).
#pragma once
#include "chem_params.cuh"
#include "newton_launch.h"
#include "newton_solve.cuh"

namespace rpb {

template <typename T, typename PR>
__device__ __forceinline__ void nt_load_fix(PR r, NtFixT<T>& F) {
    F.o2 = r[0]; F.n2 = r[1]; F.h2 = r[2]; F.co2 = r[3]; F.hnm = r[4];
    F.parthno3 = r[5]; F.parth2o = r[6]; F.parthcl = r[7]; F.parthbr = r[8];
    F.rain_hno3 = r[9]; F.rain_hcl = r[10]; F.rain_hbr = r[11]; F.rain_h2o2 = r[12]; F.dt = r[13];
}

// entry q of the queue: day cells at list[0 .. nday), night cells from the back
__device__ __forceinline__ int nt_queue_cell(const Params& P, int q, int nday) {
    return q < nday ? P.nt_list[q] : P.nt_list[P.nt_qcap - 1 - (q - nday)];
}

// The end of a lane's cell (done: iterations when converged, -1 when not):
// its status is written (a converged cell's iterations plus P.stat_bias, so
// that the write-back of the cells converged from the plain start and the
// learned restart's solve may run at the same time); the iterations of a
// cell that missed are counted.
__device__ __forceinline__ void nt_end_cell(const Params& P, int cell, int done, int it) {
    if (done < 0) atomicAdd(P.nonfinite + 5, (unsigned long long)it);  // iterations spent in vain
    P.nt_stat[cell] = done > 0 ? done + P.stat_bias : done;
}

template <typename TJ, int NTH, bool ZS>
__global__ void __launch_bounds__(NTH, 1) k_nt_solve(Params P) {
    static_assert(NTH % 32 == 0, "whole warps");
    extern __shared__ __align__(16) unsigned char nt_smem[];
    const SJ<TJ, NTH> J{reinterpret_cast<TJ*>(nt_smem) + threadIdx.x};
    const unsigned lane = threadIdx.x & 31u;
    const int nday = P.nt_head[1], nnight = P.nt_head[2];  // queue: day cells, then night cells
    const int nq = nday + nnight;
    int cell = -1;  // >= 0: cell in work; -1: wants a cell; -2: queue exhausted
    int it = 0;
    for (;;) {
        const unsigned want = __ballot_sync(0xffffffffu, cell == -1);
        if (want) {
            const int leader = __ffs(want) - 1;
            int base = 0;
            if ((int)lane == leader) base = atomicAdd(P.nt_head, __popc(want));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (cell == -1) {
                const int q = base + __popc(want & ((1u << lane) - 1u));
                cell = q < nq ? nt_queue_cell(P, q, nday) : -2;
                it = 0;
            }
        }
        if (__all_sync(0xffffffffu, cell == -2)) break;
        if (cell >= 0) {
            const double* rec = P.nt_rec + (size_t)cell * NT_REC;
            const TJ* recT;
            if constexpr (sizeof(TJ) == 4)
                recT = P.nt_rec32 + (size_t)cell * NT_REC32;
            else
                recT = rec;
            NtFixT<double> F;
            NtFixT<TJ> FT;
            nt_load_fix<double>(rec + NT_RF, F);
            nt_load_fix<TJ>(recT + NT_RF, FT);
            const bool day = rec[NT_RSZA] <= 95.;
            double* x = P.nt_x + (size_t)cell * NT_NX;
            TJ step;
            const bool ok = nt_iterate<TJ, ZS>(F, rec + NT_RK, rec + NT_RJ, rec + NT_RH, rec + NT_RCK0, FT, recT + NT_RK,
                                           recT + NT_RJ, recT + NT_RH, day, x, J, &step);
            it++;
            int done = 0;
            if (!ok)
                done = -1;
            else if (step < (TJ)P.tol)
                done = it;
            else if (it >= P.maxit)
                done = -1;
            if (done) {
                nt_end_cell(P, cell, done, it);
                cell = -1;
            }
        }
    }
}

// Two warp groups of NTH/2 lanes each take turns on one set of NTH/2 lanes'
// matrix slots. An iteration of a cell splits into a matrix phase (scaled
// Jacobian, factorisation and solve in the shared-memory slots) and an
// update phase (FP64 update with the solved step, convergence test, refill
// from the work queue, FP64 residual of the new iterate into the step
// registers z): while one group runs its matrix phase, the other runs its
// update phase, which needs no shared memory. So a block keeps NTH cells in
// flight on the shared memory of NTH/2. Phases end at a block-wide
// barrier-and-reduction that also decides, for all threads at once, when the
// queue is exhausted: every thread passes the same number of barriers, and
// none waits on another block. Phase t (t >= 1): group g runs the matrix
// phase when t + g is odd; at t = 0 group 0 runs its first update phase alone.
template <typename TJ, int NTH>
__global__ void __launch_bounds__(NTH, 1) k_nt_solve_pp(Params P) {
    constexpr int NS = NTH / 2;  // lanes of matrix slots
    static_assert(NS % 32 == 0, "whole warps per group");
    extern __shared__ __align__(16) unsigned char nt_smem[];
    const int grp = (int)threadIdx.x / NS;
    const SJ<TJ, NS> J{reinterpret_cast<TJ*>(nt_smem) + (threadIdx.x % NS)};
    const unsigned lane = threadIdx.x & 31u;
    const int nday = P.nt_head[1], nnight = P.nt_head[2];
    const int nq = nday + nnight;
    int cell = -1;  // >= 0: cell in work; -1: wants a cell; -2: queue exhausted
    int it = 0;
    bool has_z = false;  // z holds the (solved) step of the cell's current iterate
    TJ z[NT_NX];
    for (int t = 0;; t++) {
        const bool matrix_phase = ((t + grp) & 1) != 0;
        if (t == 0 && grp == 1) {
            // group 1 starts with the second phase
        } else if (!matrix_phase) {
            if (cell >= 0 && has_z) {
                const double* rec = P.nt_rec + (size_t)cell * NT_REC;
                double* x = P.nt_x + (size_t)cell * NT_NX;
                TJ step;
                const bool ok = nt_update<TJ>(x, 1e-20 * rec[NT_RF + 4], (const TJ*)z, &step, true);
                it++;
                has_z = false;
                int done = 0;
                if (!ok)
                    done = -1;
                else if (step < (TJ)P.tol)
                    done = it;
                else if (it >= P.maxit)
                    done = -1;
                if (done) {
                    nt_end_cell(P, cell, done, it);
                    cell = -1;
                }
            }
            const unsigned want = __ballot_sync(0xffffffffu, cell == -1);
            if (want) {
                const int leader = __ffs(want) - 1;
                int base = 0;
                if ((int)lane == leader) base = atomicAdd(P.nt_head, __popc(want));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (cell == -1) {
                    const int q = base + __popc(want & ((1u << lane) - 1u));
                    cell = q < nq ? nt_queue_cell(P, q, nday) : -2;
                    it = 0;
                }
            }
            if (cell >= 0) {
                const double* rec = P.nt_rec + (size_t)cell * NT_REC;
                NtFixT<double> F;
                nt_load_fix<double>(rec + NT_RF, F);
                const bool day = rec[NT_RSZA] <= 95.;
                nt_rhs<TJ>(day, F, rec + NT_RK, rec + NT_RJ, rec + NT_RH, rec + NT_RCK0,
                           (const double*)(P.nt_x + (size_t)cell * NT_NX), 1e-20 * F.hnm, (TJ*)z);
                has_z = true;
            }
        } else if (cell >= 0) {
            const double* rec = P.nt_rec + (size_t)cell * NT_REC;
            const TJ* recT;
            if constexpr (sizeof(TJ) == 4)
                recT = P.nt_rec32 + (size_t)cell * NT_REC32;
            else
                recT = rec;
            NtFixT<TJ> FT;
            nt_load_fix<TJ>(recT + NT_RF, FT);
            const bool day = rec[NT_RSZA] <= 95.;
            const double* x = P.nt_x + (size_t)cell * NT_NX;
            nt_jacobian_call<TJ>(day, FT, recT + NT_RK, recT + NT_RJ, recT + NT_RH, x, 1e-20 * rec[NT_RF + 4], J);
            NT_FENCE();
            nt_factor_solve<TJ>(J, (TJ*)z, TJ(NT_TINY));
        }
        if (__syncthreads_and(cell == -2)) break;
    }
}

// Warp-specialised form: NS cells per block, each with a matrix lane (threads
// 0..NS-1, the cell's NT_NSLOT shared-memory slots) and a residual lane
// (threads NS..2NS-1). Per iteration, phase A: the matrix lane evaluates the
// scaled Jacobian of the current iterate in TJ while the residual lane
// evaluates the FP64 residual of the same iterate into the cell's NT_NX
// right-hand-side slots (the FP32 and FP64 pipes work side by side, on the
// same cell record); phase B: the matrix lane factorises, solves, updates
// the iterate in FP64, tests convergence and refills from the work queue
// (one atomic per matrix warp), publishing the cell of the next iteration in
// shared memory. Phases end at block-wide barriers that every thread passes
// the same number of times; the exit is decided by a barrier-and-reduction
// over all threads.
template <typename T, int STRIDE>
struct SZ {
    T* p;
    __device__ __forceinline__ T& operator[](int i) const { return p[i * STRIDE]; }
};

template <typename TJ, int NS>
constexpr size_t nt_sp_smem_bytes() {
    return (size_t)(NT_NSLOT + NT_NX) * NS * sizeof(TJ) + (size_t)NS * sizeof(int);
}

template <typename TJ, int NS>
__global__ void __launch_bounds__(2 * NS, 1) k_nt_solve_sp(Params P) {
    static_assert(NS % 32 == 0, "whole warps per group");
    extern __shared__ __align__(16) unsigned char nt_smem[];
    TJ* slots = reinterpret_cast<TJ*>(nt_smem);
    int* cellbuf = reinterpret_cast<int*>(nt_smem + (size_t)(NT_NSLOT + NT_NX) * NS * sizeof(TJ));
    const bool matrix_lane = (int)threadIdx.x < NS;
    const int t = (int)threadIdx.x % NS;
    const SJ<TJ, NS> J{slots + t};
    const SZ<TJ, NS> z{slots + (size_t)NT_NSLOT * NS + t};
    const unsigned lane = threadIdx.x & 31u;
    const int nday = P.nt_head[1], nnight = P.nt_head[2];
    const int nq = nday + nnight;
    int cell = -1;  // matrix lanes: >= 0 cell in work; -1 wants a cell; -2 queue exhausted
    int it = 0;
    // the matrix warps refill their lanes and publish the cells
    auto refill = [&]() {
        const unsigned want = __ballot_sync(0xffffffffu, cell == -1);
        if (want) {
            const int leader = __ffs(want) - 1;
            int base = 0;
            if ((int)lane == leader) base = atomicAdd(P.nt_head, __popc(want));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (cell == -1) {
                const int q = base + __popc(want & ((1u << lane) - 1u));
                cell = q < nq ? nt_queue_cell(P, q, nday) : -2;
                it = 0;
            }
        }
        cellbuf[t] = cell;
    };
    if (matrix_lane) refill();
    for (;;) {
        __syncthreads();  // the published cells
        const int c = cellbuf[t];
        if (__syncthreads_and(c == -2)) break;
        // phase A
        if (c >= 0) {
            const double* rec = P.nt_rec + (size_t)c * NT_REC;
            const bool day = rec[NT_RSZA] <= 95.;
            const double* x = P.nt_x + (size_t)c * NT_NX;
            if (matrix_lane) {
                const TJ* recT;
                if constexpr (sizeof(TJ) == 4)
                    recT = P.nt_rec32 + (size_t)c * NT_REC32;
                else
                    recT = rec;
                NtFixT<TJ> FT;
                nt_load_fix<TJ>(recT + NT_RF, FT);
                nt_jacobian_call<TJ>(day, FT, recT + NT_RK, recT + NT_RJ, recT + NT_RH, x, 1e-20 * rec[NT_RF + 4], J);
            } else {
                NtFixT<double> F;
                nt_load_fix<double>(rec + NT_RF, F);
                nt_rhs<TJ>(day, F, rec + NT_RK, rec + NT_RJ, rec + NT_RH, rec + NT_RCK0, x, 1e-20 * F.hnm, z);
            }
        }
        __syncthreads();  // the Jacobian and the right-hand side of every cell
        // phase B
        if (matrix_lane) {
            if (c >= 0) {
                const double* rec = P.nt_rec + (size_t)c * NT_REC;
                double* x = P.nt_x + (size_t)c * NT_NX;
                NT_FENCE();
                nt_factor_solve<TJ>(J, z, TJ(NT_TINY));
                TJ step;
                const bool ok = nt_update<TJ>(x, 1e-20 * rec[NT_RF + 4], z, &step, true);
                it++;
                int done = 0;
                if (!ok)
                    done = -1;
                else if (step < (TJ)P.tol)
                    done = it;
                else if (it >= P.maxit)
                    done = -1;
                if (done) {
                    nt_end_cell(P, c, done, it);
                    cell = -1;
                }
            }
            refill();
        }
    }
}

// Sets the dynamic shared memory of a solve kernel and returns how many of its
// blocks an SM runs.
template <typename K>
cudaError_t nt_fit_smem(K* fn, int nthreads, size_t smem, int* blocks_per_sm) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, nthreads, smem);
}

template <typename TJ, int NS>
cudaError_t nt_sp_prepare(int* blocks_per_sm) {
    return nt_fit_smem(k_nt_solve_sp<TJ, NS>, 2 * NS, nt_sp_smem_bytes<TJ, NS>(), blocks_per_sm);
}

template <typename TJ, int NS>
cudaError_t nt_sp_launch(const Params& P, int grid, cudaStream_t stream) {
    k_nt_solve_sp<TJ, NS><<<grid, 2 * NS, nt_sp_smem_bytes<TJ, NS>(), stream>>>(P);
    return cudaGetLastError();
}

// form 3: matrix lanes and residual lanes (nth = NS cells per block)
template <typename TJ, int NS>
constexpr NtVariant nt_sp_variant() {
    return NtVariant{(int)sizeof(TJ), NS, 3, nt_sp_smem_bytes<TJ, NS>(), &nt_sp_prepare<TJ, NS>, &nt_sp_launch<TJ, NS>};
}

// Lock-step form of the one-group kernel: every warp of the block runs each
// phase of an iteration (Jacobian, residual, factorisation and solve, update
// and refill) between the same two block barriers, so that the warps of an
// SM fetch the same generated code at the same time (the solve code is far
// larger than the instruction cache). Lanes without a cell pass the barriers
// idle; the exit is a barrier-and-reduction over all threads.
template <typename TJ, int NTH>
__global__ void __launch_bounds__(NTH, 1) k_nt_solve_ls(Params P) {
    static_assert(NTH % 32 == 0, "whole warps");
    extern __shared__ __align__(16) unsigned char nt_smem[];
    const SJ<TJ, NTH> J{reinterpret_cast<TJ*>(nt_smem) + threadIdx.x};
    const unsigned lane = threadIdx.x & 31u;
    const int nday = P.nt_head[1], nnight = P.nt_head[2];
    const int nq = nday + nnight;
    int cell = -1, it = 0;
    for (;;) {
        const unsigned want = __ballot_sync(0xffffffffu, cell == -1);
        if (want) {
            const int leader = __ffs(want) - 1;
            int base = 0;
            if ((int)lane == leader) base = atomicAdd(P.nt_head, __popc(want));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (cell == -1) {
                const int q = base + __popc(want & ((1u << lane) - 1u));
                cell = q < nq ? nt_queue_cell(P, q, nday) : -2;
                it = 0;
            }
        }
        if (__syncthreads_and(cell == -2)) break;
        const double* rec = P.nt_rec + (size_t)(cell > 0 ? cell : 0) * NT_REC;
        const TJ* recT;
        if constexpr (sizeof(TJ) == 4)
            recT = P.nt_rec32 + (size_t)(cell > 0 ? cell : 0) * NT_REC32;
        else
            recT = rec;
        double* x = P.nt_x + (size_t)(cell > 0 ? cell : 0) * NT_NX;
        const bool day = rec[NT_RSZA] <= 95.;
        const double floor_ = 1e-20 * rec[NT_RF + 4];
        if (cell >= 0) {
            NtFixT<TJ> FT;
            nt_load_fix<TJ>(recT + NT_RF, FT);
            nt_jacobian_call<TJ>(day, FT, recT + NT_RK, recT + NT_RJ, recT + NT_RH, x, floor_, J);
        }
        __syncthreads();
        TJ z[NT_NX];
        if (cell >= 0) {
            NtFixT<double> F;
            nt_load_fix<double>(rec + NT_RF, F);
            nt_rhs<TJ>(day, F, rec + NT_RK, rec + NT_RJ, rec + NT_RH, rec + NT_RCK0, x, floor_, (TJ*)z);
        }
        __syncthreads();
        if (cell >= 0) {
            NT_FENCE();
            nt_factor_solve<TJ>(J, (TJ*)z, TJ(NT_TINY));
        }
        __syncthreads();
        if (cell >= 0) {
            TJ step;
            const bool ok = nt_update<TJ>(x, floor_, (const TJ*)z, &step, true);
            it++;
            int done = 0;
            if (!ok)
                done = -1;
            else if (step < (TJ)P.tol)
                done = it;
            else if (it >= P.maxit)
                done = -1;
            if (done) {
                nt_end_cell(P, cell, done, it);
                cell = -1;
            }
        }
    }
}

template <typename TJ, int NTH>
cudaError_t nt_ls_prepare(int* blocks_per_sm) {
    return nt_fit_smem(k_nt_solve_ls<TJ, NTH>, NTH, (size_t)NT_NSLOT * NTH * sizeof(TJ), blocks_per_sm);
}

template <typename TJ, int NTH>
cudaError_t nt_ls_launch(const Params& P, int grid, cudaStream_t stream) {
    k_nt_solve_ls<TJ, NTH><<<grid, NTH, (size_t)NT_NSLOT * NTH * sizeof(TJ), stream>>>(P);
    return cudaGetLastError();
}

// form 4: one group in lock-step, z in registers
template <typename TJ, int NTH>
constexpr NtVariant nt_ls_variant() {
    return NtVariant{(int)sizeof(TJ), NTH, 4, (size_t)NT_NSLOT * NTH * sizeof(TJ), &nt_ls_prepare<TJ, NTH>,
                     &nt_ls_launch<TJ, NTH>};
}

// Warps-per-cell form (form 5): W warps work on the same 32 cells. Per
// iteration, phase A: warp g of a cell group evaluates its share of the
// scaled Jacobian rows (into the cells' shared-memory matrix slots) and of the
// FP64 residual rows (scaled, into the cells' right-hand-side slots); the
// row groups are balanced by operation count at generation time and each
// evaluates only the intermediates its rows need (newton_gen.cuh,
// nt_{jacobian,residual}_{day,night}_wW). Phase B: warp 0 of the group
// factorises, solves, updates the iterate in FP64, tests convergence and
// refills its lanes from the work queue, publishing the cells of the next
// iteration. A block holds C cell groups; phases end at block barriers that
// every thread passes the same number of times, and the exit is decided by a
// barrier-and-reduction over all threads. Each warp of phase A has a smaller
// program and fewer live values than one warp evaluating every row, and an
// SM keeps W warps busy per 32 cells in flight.
template <typename TJ>
__host__ __device__ constexpr size_t nt_wc_group_bytes() {
    return (size_t)(NT_NSLOT + NT_NX) * 32 * sizeof(TJ) + 32 * sizeof(int);
}

template <int W, typename TJ, typename FFT, typename PKT, typename PJ>
__device__ __noinline__ void nt_jacobian_wc_fn(int g, bool day, const FFT& FT, PKT KT, PKT tjT, PKT hetT,
                                                const double* x, double floor_, PJ J) {
    if constexpr (W == 2) {
        if (day)
            nt_jacobian_day_w2<TJ>(g, FT, KT, tjT, hetT, x, floor_, J);
        else
            nt_jacobian_night_w2<TJ>(g, FT, KT, tjT, hetT, x, floor_, J);
    } else {
        if (day)
            nt_jacobian_day_w4<TJ>(g, FT, KT, tjT, hetT, x, floor_, J);
        else
            nt_jacobian_night_w4<TJ>(g, FT, KT, tjT, hetT, x, floor_, J);
    }
}

template <int W, typename TJ, typename FF, typename PK, typename PC, typename PZ>
__device__ __noinline__ void nt_rhs_wc_fn(int g, bool day, const FF& F, PK K, PK tj, PK het, PC ck0,
                                           const double* x, double floor_, PZ z) {
    const NtRhsOut<TJ, PZ> R{z, x, nt_exp_hi(floor_)};
    if constexpr (W == 2) {
        if (day)
            nt_residual_day_w2<double>(g, F, K, tj, het, ck0, x, R);
        else
            nt_residual_night_w2<double>(g, F, K, tj, het, ck0, x, R);
    } else {
        if (day)
            nt_residual_day_w4<double>(g, F, K, tj, het, ck0, x, R);
        else
            nt_residual_night_w4<double>(g, F, K, tj, het, ck0, x, R);
    }
}

template <typename TJ, int W, int C>
__global__ void __launch_bounds__(32 * W * C, 1) k_nt_solve_wc(Params P) {
    static_assert(W == 2 || W == 4, "row groups are generated for 2 and 4 warps per cell");
    extern __shared__ __align__(16) unsigned char nt_smem[];
    const int warp = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31u);
    const int grp = warp / W, g = warp % W;  // cell group of the block, row group of the warp
    unsigned char* base = nt_smem + (size_t)grp * nt_wc_group_bytes<TJ>();
    TJ* slots = reinterpret_cast<TJ*>(base);
    const SJ<TJ, 32> J{slots + lane};
    const SZ<TJ, 32> z{slots + (size_t)NT_NSLOT * 32 + lane};
    int* cells = reinterpret_cast<int*>(base + (size_t)(NT_NSLOT + NT_NX) * 32 * sizeof(TJ));
    const int nday = P.nt_head[1], nnight = P.nt_head[2];
    const int nq = nday + nnight;
    int cell = -1, it = 0;  // warp 0 of the group: the lane's cell and its progress
    auto refill = [&]() {
        const unsigned want = __ballot_sync(0xffffffffu, cell == -1);
        if (want) {
            const int leader = __ffs(want) - 1;
            int b = 0;
            if (lane == leader) b = atomicAdd(P.nt_head, __popc(want));
            b = __shfl_sync(0xffffffffu, b, leader);
            if (cell == -1) {
                const int q = b + __popc(want & ((1u << lane) - 1u));
                cell = q < nq ? nt_queue_cell(P, q, nday) : -2;
                it = 0;
            }
        }
        cells[lane] = cell;
    };
    if (g == 0) refill();
    for (;;) {
        __syncthreads();  // the published cells
        const int c = cells[lane];
        if (__syncthreads_and(c == -2)) break;
        const double* rec = P.nt_rec + (size_t)(c > 0 ? c : 0) * NT_REC;
        const double floor_ = 1e-20 * rec[NT_RF + 4];
        double* x = P.nt_x + (size_t)(c > 0 ? c : 0) * NT_NX;
        // phase A: this warp's rows of the Jacobian and of the residual
        if (c >= 0) {
            const TJ* recT;
            if constexpr (sizeof(TJ) == 4)
                recT = P.nt_rec32 + (size_t)c * NT_REC32;
            else
                recT = rec;
            const bool day = rec[NT_RSZA] <= 95.;
            NtFixT<TJ> FT;
            nt_load_fix<TJ>(recT + NT_RF, FT);
            if constexpr (sizeof(TJ) == 4)
                nt_jacobian_wc_fn<W, TJ>(g, day, FT, recT + NT_RK, recT + NT_RJ, recT + NT_RH, x, floor_,
                                         nt_store_view(J));
            else
                nt_jacobian_wc_fn<W, TJ>(g, day, FT, recT + NT_RK, recT + NT_RJ, recT + NT_RH, x, floor_, J);
            NtFixT<double> F;
            nt_load_fix<double>(rec + NT_RF, F);
            const SJW<TJ, 32> zw{(uint32_t)__cvta_generic_to_shared(z.p)};  // explicit shared stores
            nt_rhs_wc_fn<W, TJ>(g, day, F, rec + NT_RK, rec + NT_RJ, rec + NT_RH, rec + NT_RCK0, x, floor_, zw);
        }
        __syncthreads();  // the Jacobian and right-hand side of every cell
        // phase B: warp 0 of the group, the right-hand side in registers (the
        // factorisation's fused forward substitution reads it row by row)
        if (g == 0) {
            if (c >= 0) {
                TJ zr[NT_NX];
#pragma unroll
                for (int i = 0; i < NT_NX; i++) zr[i] = z[i];
                NT_FENCE();
                nt_factor_solve<TJ>(J, (TJ*)zr, TJ(NT_TINY));
                TJ step;
                const bool ok = nt_update<TJ>(x, floor_, (const TJ*)zr, &step, true);
                it++;
                int done = 0;
                if (!ok)
                    done = -1;
                else if (step < (TJ)P.tol)
                    done = it;
                else if (it >= P.maxit)
                    done = -1;
                if (done) {
                    nt_end_cell(P, c, done, it);
                    cell = -1;
                }
            }
            refill();
        }
    }
}

template <typename TJ, int W, int C>
cudaError_t nt_wc_prepare(int* blocks_per_sm) {
    return nt_fit_smem(k_nt_solve_wc<TJ, W, C>, 32 * W * C, C * nt_wc_group_bytes<TJ>(), blocks_per_sm);
}

template <typename TJ, int W, int C>
cudaError_t nt_wc_launch(const Params& P, int grid, cudaStream_t stream) {
    k_nt_solve_wc<TJ, W, C><<<grid, 32 * W * C, C * nt_wc_group_bytes<TJ>(), stream>>>(P);
    return cudaGetLastError();
}

// forms 5 (2 warps per cell) and 6 (4 warps per cell); nth counts the cells
// of a block (32 C)
template <typename TJ, int W, int C>
constexpr NtVariant nt_wc_variant() {
    return NtVariant{(int)sizeof(TJ), 32 * C, W == 2 ? 5 : 6, C * nt_wc_group_bytes<TJ>(), &nt_wc_prepare<TJ, W, C>,
                     &nt_wc_launch<TJ, W, C>};
}

template <typename TJ, int NTH>
constexpr size_t nt_pp_smem_bytes() {
    return (size_t)NT_NSLOT * (NTH / 2) * sizeof(TJ);
}

template <typename TJ, int NTH>
cudaError_t nt_pp_prepare(int* blocks_per_sm) {
    return nt_fit_smem(k_nt_solve_pp<TJ, NTH>, NTH, nt_pp_smem_bytes<TJ, NTH>(), blocks_per_sm);
}

template <typename TJ, int NTH>
cudaError_t nt_pp_launch(const Params& P, int grid, cudaStream_t stream) {
    k_nt_solve_pp<TJ, NTH><<<grid, NTH, nt_pp_smem_bytes<TJ, NTH>(), stream>>>(P);
    return cudaGetLastError();
}

// form 2: two warp groups sharing the matrix slots, z in registers
template <typename TJ, int NTH>
constexpr NtVariant nt_pp_variant() {
    return NtVariant{(int)sizeof(TJ), NTH, 2, nt_pp_smem_bytes<TJ, NTH>(), &nt_pp_prepare<TJ, NTH>,
                     &nt_pp_launch<TJ, NTH>};
}

template <typename TJ, int NTH, bool ZS>
constexpr size_t nt_smem_bytes() {
    return (size_t)(NT_NSLOT + (ZS ? NT_NX : 0)) * NTH * sizeof(TJ);
}

template <typename TJ, int NTH, bool ZS>
cudaError_t nt_prepare(int* blocks_per_sm) {
    return nt_fit_smem(k_nt_solve<TJ, NTH, ZS>, NTH, nt_smem_bytes<TJ, NTH, ZS>(), blocks_per_sm);
}

template <typename TJ, int NTH, bool ZS>
cudaError_t nt_launch(const Params& P, int grid, cudaStream_t stream) {
    k_nt_solve<TJ, NTH, ZS><<<grid, NTH, nt_smem_bytes<TJ, NTH, ZS>(), stream>>>(P);
    return cudaGetLastError();
}

template <typename TJ, int NTH, bool ZS>
constexpr NtVariant nt_variant() {
    return NtVariant{(int)sizeof(TJ), NTH, ZS ? 1 : 0, nt_smem_bytes<TJ, NTH, ZS>(), &nt_prepare<TJ, NTH, ZS>,
                     &nt_launch<TJ, NTH, ZS>};
}

}  // namespace rpb
