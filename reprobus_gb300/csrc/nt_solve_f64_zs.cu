// nt_solve_f64_zs.cu — FP64-matrix (plain) variants of the persistent
// Newton solve kernel, right-hand side in shared memory; the autotuner picks among the
// compiled lanes-per-block values.
#include "newton_kernel.cuh"

namespace rpb {
static const NtVariant kV[] = {nt_variant<double, 32, true>(), nt_variant<double, 64, true>()};
const NtVariant* nt_variants_f64_zs(int* n) {
    *n = (int)(sizeof(kV) / sizeof(kV[0]));
    return kV;
}
}  // namespace rpb
