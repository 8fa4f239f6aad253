// pipe_probe.cu — arithmetic-throughput probe of the GPU (FP64/FP32 FMA, FP64
// exp/log/div/sqrt, FP32 exp). Each thread writes one value to out[tid]; out
// holds exactly grid*block elements. Build: reprobus_gb300/build.py.
#include <cstdio>
#include <cuda_runtime.h>

#define CK(x) do { cudaError_t e = (x); if (e != cudaSuccess) { printf("CUDA %s at %d\n", cudaGetErrorString(e), __LINE__); return 1; } } while (0)

template <typename T>
__global__ void k_fma(T* out, int iters, T a, T b) {
    T x0 = threadIdx.x * (T)1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 16; j++) {
            x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
            x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void k_exp64(double* out, int iters) {
    double s = 0, x = -1.0 + threadIdx.x * 1e-4;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 8; j++) { s += exp(x + j * 0.01); }
        x += 1e-6;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_log64(double* out, int iters) {
    double s = 0, x = 1.0 + threadIdx.x * 1e-4;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 8; j++) { s += log(x + j * 0.01); }
        x += 1e-6;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_div64(double* out, int iters) {
    double s = 0, x = 1.0 + threadIdx.x * 1e-4;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 8; j++) { s += 1.7 / (x + j * 0.01); }
        x += 1e-6;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_sqrt64(double* out, int iters) {
    double s = 0, x = 1.0 + threadIdx.x * 1e-4;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 8; j++) { s += sqrt(x + j * 0.01); }
        x += 1e-6;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_exp32(float* out, int iters) {
    float s = 0, x = -1.0f + threadIdx.x * 1e-4f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 8; j++) { s += expf(x + j * 0.01f); }
        x += 1e-6f;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int main() {
    int dev = 0, nsm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    cudaDeviceProp pr;
    CK(cudaGetDeviceProperties(&pr, dev));
    printf("device %s sms %d cc %d.%d\n", pr.name, nsm, pr.major, pr.minor);
    const int block = 256, grid = nsm * 8;
    const size_t n = (size_t)grid * block;
    double* d64; float* d32;
    CK(cudaMalloc(&d64, n * sizeof(double)));
    CK(cudaMalloc(&d32, n * sizeof(float)));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0)); CK(cudaEventCreate(&e1));
    float ms;
    for (int rep = 0; rep < 2; rep++) {
        int it = 2000;
        CK(cudaEventRecord(e0));
        k_fma<double><<<grid, block>>>(d64, it, 0.999999, 1e-7);
        CK(cudaEventRecord(e1)); CK(cudaEventSynchronize(e1)); CK(cudaGetLastError());
        CK(cudaEventElapsedTime(&ms, e0, e1));
        double ops = (double)n * it * 16 * 8;
        printf("DFMA: %.3f ms  %.3f TFMA/s = %.3f TFLOP/s\n", ms, ops / ms / 1e9, 2 * ops / ms / 1e9);
        it = 20000;
        CK(cudaEventRecord(e0));
        k_fma<float><<<grid, block>>>(d32, it, 0.999999f, 1e-7f);
        CK(cudaEventRecord(e1)); CK(cudaEventSynchronize(e1)); CK(cudaGetLastError());
        CK(cudaEventElapsedTime(&ms, e0, e1));
        ops = (double)n * it * 16 * 8;
        printf("FFMA: %.3f ms  %.3f TFMA/s = %.3f TFLOP/s\n", ms, ops / ms / 1e9, 2 * ops / ms / 1e9);
        it = 200;
        CK(cudaEventRecord(e0)); k_exp64<<<grid, block>>>(d64, it); CK(cudaEventRecord(e1)); CK(cudaEventSynchronize(e1)); CK(cudaGetLastError());
        CK(cudaEventElapsedTime(&ms, e0, e1)); printf("exp64: %.3f ms  %.3f Gexp/s\n", ms, (double)n * it * 8 / ms / 1e6);
        CK(cudaEventRecord(e0)); k_log64<<<grid, block>>>(d64, it); CK(cudaEventRecord(e1)); CK(cudaEventSynchronize(e1)); CK(cudaGetLastError());
        CK(cudaEventElapsedTime(&ms, e0, e1)); printf("log64: %.3f ms  %.3f Glog/s\n", ms, (double)n * it * 8 / ms / 1e6);
        CK(cudaEventRecord(e0)); k_div64<<<grid, block>>>(d64, it); CK(cudaEventRecord(e1)); CK(cudaEventSynchronize(e1)); CK(cudaGetLastError());
        CK(cudaEventElapsedTime(&ms, e0, e1)); printf("div64: %.3f ms  %.3f Gdiv/s\n", ms, (double)n * it * 8 / ms / 1e6);
        CK(cudaEventRecord(e0)); k_sqrt64<<<grid, block>>>(d64, it); CK(cudaEventRecord(e1)); CK(cudaEventSynchronize(e1)); CK(cudaGetLastError());
        CK(cudaEventElapsedTime(&ms, e0, e1)); printf("sqrt64: %.3f ms  %.3f Gsqrt/s\n", ms, (double)n * it * 8 / ms / 1e6);
        it = 2000;
        CK(cudaEventRecord(e0)); k_exp32<<<grid, block>>>(d32, it); CK(cudaEventRecord(e1)); CK(cudaEventSynchronize(e1)); CK(cudaGetLastError());
        CK(cudaEventElapsedTime(&ms, e0, e1)); printf("exp32: %.3f ms  %.3f Gexp/s\n", ms, (double)n * it * 8 / ms / 1e6);
    }
    CK(cudaFree(d64)); CK(cudaFree(d32));
    return 0;
}
