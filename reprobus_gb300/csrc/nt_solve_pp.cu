// nt_solve_pp.cu — variants of the persistent Newton solve kernel in which two
// warp groups take turns on one set of matrix slots (k_nt_solve_pp): FP32
// matrices (mixed solver) and FP64 matrices (plain solver); the autotuner picks
// among them and the one-group variants.
#include "newton_kernel.cuh"

namespace rpb {
static const NtVariant kF32[] = {nt_pp_variant<float, 128>(), nt_pp_variant<float, 256>()};
static const NtVariant kF64[] = {nt_pp_variant<double, 64>(), nt_pp_variant<double, 128>()};
const NtVariant* nt_variants_f32_pp(int* n) {
    *n = (int)(sizeof(kF32) / sizeof(kF32[0]));
    return kF32;
}
const NtVariant* nt_variants_f64_pp(int* n) {
    *n = (int)(sizeof(kF64) / sizeof(kF64[0]));
    return kF64;
}
}  // namespace rpb
