// Device build of the generated equations' quotients and pivot reciprocals
// (nt_div, nt_rcp in reprobus_gb300/csrc/newton_num.cuh) beside the IEEE
// operations, for tests/test_gpu_div64.py.
#include <cuda_runtime.h>

#include "../reprobus_gb300/csrc/newton_num.cuh"

__global__ void k_nt_div(const double* a, const double* b, const float* af, const float* bf, double* qd,
                         double* ieee, float* qf, float* rf, long n) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    qd[i] = rpb::nt_div<double>(a[i], b[i]);
    ieee[i] = a[i] / b[i];
    qf[i] = rpb::nt_div<float>(af[i], bf[i]);
    rf[i] = rpb::nt_rcp<float>(bf[i]);
}

// host arrays a, b (FP64) and af, bf (FP32), n each -> qd = nt_div<double>,
// ieee = a / b, qf = nt_div<float>, rf = nt_rcp<float>(bf); returns a cudaError_t
extern "C" int nt_div_dev(const double* a, const double* b, const float* af, const float* bf, double* qd,
                          double* ieee, float* qf, float* rf, long n) {
    void* d[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    const size_t b8 = (size_t)n * sizeof(double), b4 = (size_t)n * sizeof(float);
    const size_t sz[8] = {b8, b8, b4, b4, b8, b8, b4, b4};
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 8 && !e; k++) e = cudaMalloc(&d[k], sz[k]);
    if (!e) e = cudaMemcpy(d[0], a, b8, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(d[1], b, b8, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(d[2], af, b4, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(d[3], bf, b4, cudaMemcpyHostToDevice);
    if (!e) {
        k_nt_div<<<(unsigned)((n + 255) / 256), 256>>>((const double*)d[0], (const double*)d[1], (const float*)d[2],
                                                       (const float*)d[3], (double*)d[4], (double*)d[5],
                                                       (float*)d[6], (float*)d[7], n);
        e = cudaGetLastError();
    }
    if (!e) e = cudaMemcpy(qd, d[4], b8, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(ieee, d[5], b8, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(qf, d[6], b4, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(rf, d[7], b4, cudaMemcpyDeviceToHost);
    for (int k = 0; k < 8; k++) cudaFree(d[k]);
    return (int)e;
}
