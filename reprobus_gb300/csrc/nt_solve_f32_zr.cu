// nt_solve_f32_zr.cu — FP32-matrix (mixed-precision) variants of the persistent
// Newton solve kernel, right-hand side in registers; the autotuner picks among the
// compiled lanes-per-block values.
#include "newton_kernel.cuh"

namespace rpb {
static const NtVariant kV[] = {nt_variant<float, 64, false>(), nt_variant<float, 96, false>(), nt_variant<float, 128, false>()};
const NtVariant* nt_variants_f32_zr(int* n) {
    *n = (int)(sizeof(kV) / sizeof(kV[0]));
    return kV;
}
}  // namespace rpb
