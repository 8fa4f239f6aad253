// newton_launch.h — the compiled variants of the persistent Newton solve
// kernel (newton_kernel.cuh), as seen by the step code in chem_kernels.cu.
#pragma once
#include <cuda_runtime.h>

namespace rpb {
struct Params;

struct NtVariant {
    int tj_bytes;  // matrix precision: 4 = FP32 (mixed solver), 8 = FP64 (plain solver)
    int nth;       // lanes per block = cells in flight per block
    int zshared;   // 1: right-hand side / step in shared memory, 0: in registers,
                   // 2: in registers, two warp groups taking turns on the matrix slots,
                   // 3: in shared memory, written by a residual lane per cell,
                   // 4: in registers, the block's warps in lock-step,
                   // 5, 6: in shared memory, 2 or 4 warps per cell (nth: cells per block)
    size_t smem;   // dynamic shared memory per block (the cells' matrix slots)
    cudaError_t (*prepare)(int* blocks_per_sm);  // shared-memory opt-in, occupancy
    cudaError_t (*launch)(const Params& P, int grid, cudaStream_t stream);
};

// variants compiled in nt_solve_{f32,f64}_{zr,zs}.cu, nt_solve_{pp,sp,ls,wc}.cu,
// gathered in chem_kernels.cu: the matrix precision's variants, z in
// registers first
const NtVariant* nt_variants_f32_zr(int* n);
const NtVariant* nt_variants_f32_zs(int* n);
const NtVariant* nt_variants_f64_zr(int* n);
const NtVariant* nt_variants_f64_zs(int* n);
const NtVariant* nt_variants_f32_pp(int* n);
const NtVariant* nt_variants_f64_pp(int* n);
const NtVariant* nt_variants_f32_sp(int* n);
const NtVariant* nt_variants_f64_sp(int* n);
const NtVariant* nt_variants_f32_ls(int* n);
const NtVariant* nt_variants_f64_ls(int* n);
const NtVariant* nt_variants_f32_wc(int* n);
const NtVariant* nt_variants_f64_wc(int* n);
}  // namespace rpb
