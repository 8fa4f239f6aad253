// nt_solve_ls.cu — lock-step variants of the one-group persistent Newton
// solve kernel (k_nt_solve_ls), FP32 and FP64 matrices; the autotuner picks
// among them and the other forms.
#include "newton_kernel.cuh"

namespace rpb {
static const NtVariant kF32[] = {nt_ls_variant<float, 64>(), nt_ls_variant<float, 128>()};
static const NtVariant kF64[] = {nt_ls_variant<double, 32>(), nt_ls_variant<double, 64>()};
const NtVariant* nt_variants_f32_ls(int* n) {
    *n = (int)(sizeof(kF32) / sizeof(kF32[0]));
    return kF32;
}
const NtVariant* nt_variants_f64_ls(int* n) {
    *n = (int)(sizeof(kF64) / sizeof(kF64[0]));
    return kF64;
}
}  // namespace rpb
