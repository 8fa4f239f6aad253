// mlp_net.h — what the chemistry step code (chem_kernels.cu) sees of the
// network of the learned restart (mlp_kernels.cu).
#pragma once
#include <cuda_runtime.h>

namespace rpb {
constexpr int MLP_FEAT = 64;  // features per cell (raw, FP32)
constexpr int MLP_YOUT = 64;  // outputs per cell (raw log10 end-of-step ratios, 57 used)
// cells of one step that the learned restart takes at most (the others fall back)
constexpr int MLP_RESTART_CAP = 65536;
// whole network on B rows of raw features X -> raw outputs Y (device arrays);
// with rows_dev, on min(B, *rows_dev) rows (a count the device wrote)
int mlp_infer(void* net, const float* X, float* Y, int B, cudaStream_t s, const int* rows_dev = nullptr);
unsigned int* mlp_err_flag(void* net);
int mlp_fail(const char* what, cudaError_t e, int line);
}  // namespace rpb

// sets the calling thread's error text (chem_kernels.cu); returns code
extern "C" __attribute__((visibility("hidden"))) int reprobus_set_error(int code, const char* fmt, ...);
