// Host build of log64 (reprobus_gb300/csrc/log64.cuh) for the CPU checks of
// tests/test_log64.py (compiled with -ffp-contract=off: the device code's
// fused multiply-adds and nothing else fused).
#include "../reprobus_gb300/csrc/log64.cuh"

extern "C" void log64_many(const double* x, double* out, long n) {
    for (long i = 0; i < n; i++) out[i] = rpb::log64(x[i]);
}
