// Host build of div64 (reprobus_gb300/csrc/div64.cuh) for the CPU checks of
// tests/test_div64.py (compiled with -ffp-contract=off: the same fused
// multiply-adds as the device code; the host's reciprocal estimate is 1 / b
// rounded down to 20 bits).
#include "../reprobus_gb300/csrc/div64.cuh"

extern "C" void div64_many(const double* a, const double* b, double* out, long n) {
    for (long i = 0; i < n; i++) out[i] = rpb::div64(a[i], b[i]);
}

extern "C" void sqrt64_many(const double* x, double* out, long n) {
    for (long i = 0; i < n; i++) out[i] = rpb::sqrt64(x[i]);
}
