// Device build of exp64 (reprobus_gb300/csrc/exp64.cuh) beside CUDA's exp,
// for tests/test_gpu_exp64.py: both over the same arguments, in one kernel.
#include <cuda_runtime.h>

#include "../reprobus_gb300/csrc/exp64.cuh"

__global__ void k_exp64(const double* y, double* a, double* b, long n) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    a[i] = rpb::exp64(y[i]);
    b[i] = exp(y[i]);
}

// host arrays y[n] -> a[n] (exp64), b[n] (CUDA exp); returns a cudaError_t
extern "C" int exp64_dev(const double* y, double* a, double* b, long n) {
    double *dy = nullptr, *da = nullptr, *db = nullptr;
    const size_t bytes = (size_t)n * sizeof(double);
    cudaError_t e = cudaMalloc(&dy, bytes);
    if (!e) e = cudaMalloc(&da, bytes);
    if (!e) e = cudaMalloc(&db, bytes);
    if (!e) e = cudaMemcpy(dy, y, bytes, cudaMemcpyHostToDevice);
    if (!e) {
        k_exp64<<<(unsigned)((n + 255) / 256), 256>>>(dy, da, db, n);
        e = cudaGetLastError();
    }
    if (!e) e = cudaMemcpy(a, da, bytes, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(b, db, bytes, cudaMemcpyDeviceToHost);
    cudaFree(dy);
    cudaFree(da);
    cudaFree(db);
    return (int)e;
}
