// nt_solve_sp.cu — warp-specialised variants of the persistent Newton solve
// kernel (k_nt_solve_sp: a matrix lane and a residual lane per cell), FP32
// matrices (mixed solver) and FP64 matrices (plain solver); the autotuner
// picks among them and the other forms.
#include "newton_kernel.cuh"

namespace rpb {
static const NtVariant kF32[] = {nt_sp_variant<float, 64>(), nt_sp_variant<float, 128>()};
static const NtVariant kF64[] = {nt_sp_variant<double, 32>(), nt_sp_variant<double, 64>()};
const NtVariant* nt_variants_f32_sp(int* n) {
    *n = (int)(sizeof(kF32) / sizeof(kF32[0]));
    return kF32;
}
const NtVariant* nt_variants_f64_sp(int* n) {
    *n = (int)(sizeof(kF64) / sizeof(kF64[0]));
    return kF64;
}
}  // namespace rpb
