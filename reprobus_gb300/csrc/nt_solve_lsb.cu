// nt_solve_lsb.cu — the lock-step solve kernel with its FP32 matrix slots
// stored as BF16 (k_nt_solve_ls<float, NTH, true>): half the shared memory per
// cell, so up to twice the cells in flight per SM; an autotuner candidate of
// the mixed solver (its own translation unit so that nvcc builds it in
// parallel with the others).
#include "newton_kernel.cuh"

namespace rpb {
static const NtVariant kF32[] = {nt_lsb_variant<64>(), nt_lsb_variant<128>(), nt_lsb_variant<256>()};
const NtVariant* nt_variants_f32_lsb(int* n) {
    *n = (int)(sizeof(kF32) / sizeof(kF32[0]));
    return kF32;
}
}  // namespace rpb
