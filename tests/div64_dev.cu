// Device build of div64 (reprobus_gb300/csrc/div64.cuh) beside the IEEE
// division, for tests/test_gpu_div64.py.
#include <cuda_runtime.h>

#include "../reprobus_gb300/csrc/div64.cuh"

__global__ void k_div64(const double* a, const double* b, double* q, double* ieee, long n) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    q[i] = rpb::div64(a[i], b[i]);
    ieee[i] = a[i] / b[i];
}

__global__ void k_sqrt64(const double* x, double* q, double* ieee, long n) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    q[i] = rpb::sqrt64(x[i]);
    ieee[i] = sqrt(x[i]);
}

// host arrays a[n], b[n] -> q[n] (div64), ieee[n] (a / b); returns a cudaError_t
extern "C" int div64_dev(const double* a, const double* b, double* q, double* ieee, long n) {
    double *d[4] = {nullptr, nullptr, nullptr, nullptr};
    const size_t bytes = (size_t)n * sizeof(double);
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 4 && !e; k++) e = cudaMalloc(&d[k], bytes);
    if (!e) e = cudaMemcpy(d[0], a, bytes, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(d[1], b, bytes, cudaMemcpyHostToDevice);
    if (!e) {
        k_div64<<<(unsigned)((n + 255) / 256), 256>>>(d[0], d[1], d[2], d[3], n);
        e = cudaGetLastError();
    }
    if (!e) e = cudaMemcpy(q, d[2], bytes, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(ieee, d[3], bytes, cudaMemcpyDeviceToHost);
    for (int k = 0; k < 4; k++) cudaFree(d[k]);
    return (int)e;
}

// host arrays x[n] -> q[n] (sqrt64), ieee[n] (sqrt); returns a cudaError_t
extern "C" int sqrt64_dev(const double* x, double* q, double* ieee, long n) {
    double *d[3] = {nullptr, nullptr, nullptr};
    const size_t bytes = (size_t)n * sizeof(double);
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 3 && !e; k++) e = cudaMalloc(&d[k], bytes);
    if (!e) e = cudaMemcpy(d[0], x, bytes, cudaMemcpyHostToDevice);
    if (!e) {
        k_sqrt64<<<(unsigned)((n + 255) / 256), 256>>>(d[0], d[1], d[2], n);
        e = cudaGetLastError();
    }
    if (!e) e = cudaMemcpy(q, d[1], bytes, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(ieee, d[2], bytes, cudaMemcpyDeviceToHost);
    for (int k = 0; k < 3; k++) cudaFree(d[k]);
    return (int)e;
}
