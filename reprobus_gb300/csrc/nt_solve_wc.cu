// nt_solve_wc.cu — warps-per-cell variants of the persistent Newton solve
// kernel (k_nt_solve_wc): 2 or 4 warps share 32 cells, in blocks of one or
// two such groups, FP32 and FP64 matrices; the autotuner picks among them and
// the other forms.
#include "newton_kernel.cuh"

namespace rpb {
static const NtVariant kF32[] = {nt_wc_variant<float, 2, 1>(), nt_wc_variant<float, 2, 2>(),
                                 nt_wc_variant<float, 4, 1>()};
static const NtVariant kF64[] = {nt_wc_variant<double, 2, 1>(), nt_wc_variant<double, 4, 1>()};
const NtVariant* nt_variants_f32_wc(int* n) {
    *n = (int)(sizeof(kF32) / sizeof(kF32[0]));
    return kF32;
}
const NtVariant* nt_variants_f64_wc(int* n) {
    *n = (int)(sizeof(kF64) / sizeof(kF64[0]));
    return kF64;
}
}  // namespace rpb
