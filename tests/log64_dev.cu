// Device build of log64 (reprobus_gb300/csrc/log64.cuh) beside CUDA's log,
// for tests/test_gpu_log64.py: both over the same arguments, in one kernel.
#include <cuda_runtime.h>

#include "../reprobus_gb300/csrc/log64.cuh"

__global__ void k_log64(const double* x, double* a, double* b, long n) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    a[i] = rpb::log64(x[i]);
    b[i] = log(x[i]);
}

// host arrays x[n] -> a[n] (log64), b[n] (CUDA log); returns a cudaError_t
extern "C" int log64_dev(const double* x, double* a, double* b, long n) {
    double *dx = nullptr, *da = nullptr, *db = nullptr;
    const size_t bytes = (size_t)n * sizeof(double);
    cudaError_t e = cudaMalloc(&dx, bytes);
    if (!e) e = cudaMalloc(&da, bytes);
    if (!e) e = cudaMalloc(&db, bytes);
    if (!e) e = cudaMemcpy(dx, x, bytes, cudaMemcpyHostToDevice);
    if (!e) {
        k_log64<<<(unsigned)((n + 255) / 256), 256>>>(dx, da, db, n);
        e = cudaGetLastError();
    }
    if (!e) e = cudaMemcpy(a, da, bytes, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(b, db, bytes, cudaMemcpyDeviceToHost);
    cudaFree(dx);
    cudaFree(da);
    cudaFree(db);
    return (int)e;
}
