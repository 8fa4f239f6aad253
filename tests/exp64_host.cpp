// Host build of exp64 (reprobus_gb300/csrc/exp64.cuh) for the CPU checks of
// tests/test_exp64.py. Compiled with -ffp-contract=off, so that its
// arithmetic is the device code's: the same FP64 and FP32 fused multiply-adds
// and integer operations, each rounded once.
#include "../reprobus_gb300/csrc/exp64.cuh"

extern "C" void exp64_many(const double* y, double* out, long n) {
    for (long i = 0; i < n; i++) out[i] = rpb::exp64(y[i]);
}
