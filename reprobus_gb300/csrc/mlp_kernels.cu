// mlp_kernels.cu — the network of the Newton solvers' learned restart (the
// start of the cells whose plain start misses): a 64-256-256-256-64 MLP
// (SiLU) with BF16 weights and activations and FP32 accumulation on the
// tcgen05 tensor cores, trained on the GPU by these kernels.
//
//   k_gemm_tn<EPI>   C[M x N] = A[M x K] B[N x K]^T, one 128 x BN tile per CTA,
//                    K in chunks of 64 staged in shared memory (tc_sm100.cuh
//                    layout), accumulator in TMEM; epilogues: plain FP32,
//                    forward layer (bias, SiLU, BF16 copy), backward through
//                    SiLU (BF16 gradient of the previous layer)
//   k_mlp_infer      the whole network for 128 cells per tile, persistent:
//                    activations stay in shared memory, weights stream from L2
//   k_transpose_bf16, k_loss, k_colsum, k_adam   training helpers
//
// Sizes: M multiple of 128, N multiple of 16 up to 256, K multiple of 64.
// Every mbarrier wait is bounded; a wait that gives up sets an error flag
// (reported as REPROBUS_ERR_TIMEOUT) and the kernel skips the rest of its work.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "tc_sm100.cuh"

namespace rpb {

constexpr uint32_t MB_POLLS = 1u << 24;  // mbarrier polls before a wait gives up

enum { EPI_F32 = 0, EPI_FWD = 1, EPI_BWD_SILU = 2 };

struct GemmArgs {
    const __nv_bfloat16* A;  // M x K, row-major (K contiguous)
    const __nv_bfloat16* B;  // N x K, row-major
    int M, N, K;
    float* C;                // EPI_F32: M x N FP32 (ldc = N); EPI_FWD: pre-activation Z (ldc = N)
    const float* bias;       // EPI_FWD: N
    __nv_bfloat16* H;        // EPI_FWD: SiLU(Z) BF16 (ld = N); EPI_BWD_SILU: dZprev BF16 (ld = N)
    const float* Zprev;      // EPI_BWD_SILU: pre-activation of the previous layer (M x N)
    int act;                 // EPI_FWD: 1 = SiLU, 0 = identity
    unsigned int* err;
};

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }
// SiLU for the inference epilogues, whose results are rounded to BF16:
// z sigmoid(z) = z (1 + tanh(z / 2)) / 2 with the hardware tanh approximation
// (one MUFU instruction, error far below the BF16 rounding of the result)
__device__ __forceinline__ float silu_bf(float z) {
    float t;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(0.5f * z));
    return 0.5f * z * (1.f + t);
}
__device__ __forceinline__ float dsilu(float z) {
    const float s = 1.f / (1.f + __expf(-z));
    return s * (1.f + z * (1.f - s));
}

// copy a rows x 64 BF16 chunk (row stride ld elements, starting column k0)
// into the K-major core-matrix layout (kdim 64); rows past nrows are zero
__device__ __forceinline__ void stage_chunk(uint8_t* dst, const __nv_bfloat16* src, int rows, int nrows, int ld,
                                            int k0) {
    for (int i = threadIdx.x; i < rows * 8; i += blockDim.x) {
        const int r = i >> 3, k8 = i & 7;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (r < nrows) v = *reinterpret_cast<const uint4*>(src + (size_t)r * ld + k0 + k8 * 8);
        *reinterpret_cast<uint4*>(dst + tc_off(r, k8 * 8, 64)) = v;
    }
}

template <int EPI, int BN>
__global__ void __launch_bounds__(128) k_gemm_tn(GemmArgs g) {
    extern __shared__ __align__(1024) uint8_t sm[];
    uint8_t* As = sm;                    // 128 x 64 BF16 = 16 KB
    uint8_t* Bs = sm + 128 * 64 * 2;     // BN x 64 BF16
    __shared__ uint64_t bar;
    __shared__ uint32_t tslot;
    const int m0 = blockIdx.x * 128, n0 = blockIdx.y * BN;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) tmem_alloc(&tslot, BN < 32 ? 32 : BN);
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tslot;
    uint32_t phase = 0;
    bool ok = true;
    const uint32_t idesc = tc_idesc_bf16(128, BN);
    for (int k0 = 0; k0 < g.K && ok; k0 += 64) {
        stage_chunk(As, g.A + (size_t)m0 * g.K, 128, g.M - m0, g.K, k0);
        stage_chunk(Bs, g.B + (size_t)n0 * g.K, BN, g.N - n0, g.K, k0);
        fence_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            tc_fence_after();
#pragma unroll
            for (int kk = 0; kk < 4; kk++) {
                const uint64_t ad = tc_desc(smem_u32(As) + kk * 256, 128, 64 / 8 * 128);
                const uint64_t bd = tc_desc(smem_u32(Bs) + kk * 256, 128, 64 / 8 * 128);
                tc_mma_bf16(tbase, ad, bd, idesc, k0 > 0 || kk > 0);
            }
            tc_commit(&bar);
        }
        ok = mbar_wait(&bar, phase, MB_POLLS);  // the MMAs are done: the chunk buffers may be rewritten
        ok = __syncthreads_and(ok);             // one verdict for the block (and the barrier before that)
        if (ok) phase ^= 1;
    }
    tc_fence_after();
    if (!ok) {
        // the wait gave up: the MMAs of the outstanding phase get a last
        // bounded chance to finish before TMEM is released
        mbar_wait(&bar, phase, MB_POLLS);
        if (threadIdx.x == 0) atomicAdd(g.err, 1u);
    } else {
        const int row = m0 + warp * 32 + lane;
        const uint32_t trow = tbase + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int c = 0; c < BN; c += 16) {
            float v[16];
            tmem_ld16(trow + c, v);
            if (row < g.M) {
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int col = n0 + c + j;
                    if (col >= g.N) continue;
                    const size_t o = (size_t)row * g.N + col;
                    if (EPI == EPI_F32) {
                        g.C[o] = v[j];
                    } else if (EPI == EPI_FWD) {
                        const float z = v[j] + g.bias[col];
                        g.C[o] = z;
                        g.H[o] = __float2bfloat16(g.act ? silu(z) : z);
                    } else {
                        g.H[o] = __float2bfloat16(v[j] * dsilu(g.Zprev[o]));
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tbase, BN < 32 ? 32 : BN);
}


// ---------------------------------------------------------------------------
// network shape: 64 -> 256 -> 256 -> 256 -> 64, SiLU after the hidden layers
// ---------------------------------------------------------------------------
constexpr int MLP_NL = 4;
constexpr int MLP_IN = 64;    // 57 log10 mixing ratios + T, ln p, cos sza, log10 aerosol area, lat, time of day, 0
constexpr int MLP_H = 256;
constexpr int MLP_OUT = 64;   // 57 log10 end-of-step ratios + 7 padding outputs (zero weight in the loss)
constexpr int MLP_NY = 57;
__host__ __device__ constexpr int mlp_fan_in(int l) { return l == 0 ? MLP_IN : MLP_H; }
__host__ __device__ constexpr int mlp_fan_out(int l) { return l == MLP_NL - 1 ? MLP_OUT : MLP_H; }
constexpr int MLP_K0 = 2 * MLP_IN;  // layer 0 sees each normalised feature as a BF16 pair hi + lo
                                    // (hi = bf16(x), lo = bf16(x - hi)): ~16 mantissa bits of input
constexpr int MLP_NPARAM = MLP_IN * MLP_H + MLP_H + 2 * (MLP_H * MLP_H + MLP_H) + MLP_H * MLP_OUT + MLP_OUT;
constexpr int MLP_NNORM = 2 * MLP_IN + 3 * MLP_OUT;  // in_mean, in_std, out_mean, out_std, out_min
// out_min: per output, the smallest |prediction| that is applied (smaller
// predicted corrections are replaced by 0: the plain start is kept)

// the weights of one inference tile as six shared-memory images in the
// core-matrix layout, stored back to back in global memory so that each one
// is a single bulk (TMA) copy: [W0 | W0] (256 x 128), W1 rows 0-127 and
// 128-255, W2 rows 0-127 and 128-255 (128 x 256 each), W3 (64 x 256)
constexpr int WIMG_N = 6;
__host__ __device__ constexpr uint32_t wimg_bytes(int i) { return i == WIMG_N - 1 ? 32768u : 65536u; }
__host__ __device__ constexpr uint32_t wimg_off(int i) { return (uint32_t)i * 65536u; }
constexpr uint32_t WIMG_TOTAL = 5 * 65536 + 32768;

struct InferArgs {
    const float* X;              // B x 64 raw features
    float* Y;                    // B x 64 raw outputs (log10 corrections)
    int B;
    const int* Bdev;             // set: rows = min(B, *Bdev), a count written on the device
    const uint8_t* img;          // WIMG_TOTAL bytes of weight images
    const float* b[MLP_NL];
    const float* norm;
    unsigned int* err;
    uint32_t polls;              // polls before a wait on a weight image or the MMAs gives up
};

// build the weight images from the BF16 row-major weights
__global__ void k_wimage(const __nv_bfloat16* W0c, const __nv_bfloat16* W1, const __nv_bfloat16* W2,
                         const __nv_bfloat16* W3, uint8_t* img) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;  // one 16-byte chunk (8 elements)
    // image 0: 256 x 128 (16 chunks per row)
    if (i < 256 * 16) {
        const int r = i / 16, k8 = i % 16;
        *reinterpret_cast<uint4*>(img + wimg_off(0) + tc_off(r, k8 * 8, MLP_K0)) =
            *reinterpret_cast<const uint4*>(W0c + (size_t)r * MLP_K0 + k8 * 8);
        return;
    }
    int j = i - 256 * 16;
    // images 1-4: 128 x 256 halves (32 chunks per row)
    if (j < 4 * 128 * 32) {
        const int im = j / (128 * 32), rem = j % (128 * 32), r = rem / 32, k8 = rem % 32;
        const __nv_bfloat16* W = im < 2 ? W1 : W2;
        const int row = (im & 1) * 128 + r;
        *reinterpret_cast<uint4*>(img + wimg_off(1 + im) + tc_off(r, k8 * 8, MLP_H)) =
            *reinterpret_cast<const uint4*>(W + (size_t)row * MLP_H + k8 * 8);
        return;
    }
    j -= 4 * 128 * 32;
    // image 5: 64 x 256
    if (j < 64 * 32) {
        const int r = j / 32, k8 = j % 32;
        *reinterpret_cast<uint4*>(img + wimg_off(5) + tc_off(r, k8 * 8, MLP_H)) =
            *reinterpret_cast<const uint4*>(W3 + (size_t)r * MLP_H + k8 * 8);
    }
}
constexpr int WIMG_CHUNKS = 256 * 16 + 4 * 128 * 32 + 64 * 32;

// the whole network on 128 rows per tile (persistent over tiles): input
// normalisation, 4 layers on the tensor cores with the activations kept in
// shared memory, output de-normalisation. The six weight images of a tile
// stream through two 64 KB buffers by bulk copies: the copy of the next
// image runs while the tensor cores work on the current one. 8 warps: warps
// w and w + 4 read the same TMEM lane quarter (rows 32 (w % 4) ..) and split
// the accumulator columns between them in the epilogues.
constexpr int MLP_INFER_THREADS = 256;
__global__ void __launch_bounds__(MLP_INFER_THREADS, 1) k_mlp_infer(InferArgs a) {
    extern __shared__ __align__(1024) uint8_t sm[];
    uint8_t* act = sm;                                     // 128 x 256 BF16 (64 KB)
    uint8_t* wbuf[2] = {sm + 65536, sm + 131072};          // weight images (64 KB each)
    float* bias = reinterpret_cast<float*>(sm + 196608);   // 832 floats
    float* nrm = bias + 3 * MLP_H + MLP_OUT;               // MLP_NNORM floats
    __shared__ uint64_t bar, wbar[2];
    __shared__ uint32_t tslot;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (a.Bdev) a.B = min(a.B, max(*a.Bdev, 0));
    const int ntiles = (a.B + 127) / 128;
    const int my_tiles = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const int nimg = my_tiles * WIMG_N;  // weight images this CTA loads in all
    if (warp == 0) tmem_alloc(&tslot, 256);
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_init(&wbar[0], 1);
        mbar_init(&wbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int i = threadIdx.x; i < MLP_H; i += blockDim.x) {
        bias[i] = a.b[0][i];
        bias[MLP_H + i] = a.b[1][i];
        bias[2 * MLP_H + i] = a.b[2][i];
    }
    for (int i = threadIdx.x; i < MLP_OUT; i += blockDim.x) bias[3 * MLP_H + i] = a.b[3][i];
    // the input standard deviations as reciprocals (a product per feature)
    for (int i = threadIdx.x; i < MLP_NNORM; i += blockDim.x)
        nrm[i] = (i >= MLP_IN && i < 2 * MLP_IN) ? 1.f / a.norm[i] : a.norm[i];
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tslot;
    const int quarter = warp & 3, chalf = warp >> 2;  // TMEM lane quarter, column half
    const uint32_t trow = tbase + ((uint32_t)(quarter * 32) << 16);
    // Phases are consumed only by waits that succeed: after a wait gives up,
    // wph/phase still name the phase that is outstanding, and pend/mpend say
    // whether a copy (per buffer) or the MMAs are still in flight, so that
    // the exit path waits for exactly those before it frees TMEM. ok is
    // block-uniform (each verdict goes through __syncthreads_and), so every
    // thread keeps the same bookkeeping.
    uint32_t phase = 0, wph[2] = {0, 0};
    bool pend[2] = {nimg > 0, false}, mpend = false;
    bool ok = true;
    if (threadIdx.x == 0 && nimg > 0) {
        mbar_expect_tx(&wbar[0], wimg_bytes(0));
        bulk_g2s(wbuf[0], a.img + wimg_off(0), wimg_bytes(0), &wbar[0]);
    }
    int q = 0;  // weight images consumed so far
    // MMAs of weight image q % WIMG_N (in wbuf[q & 1]) into TMEM columns
    // [dcol, dcol + N); the copy of image q + 1 starts once they are issued
    auto mma_img = [&](uint32_t dcol, int K, int N) {
        const int buf = q & 1;
        fence_async_smem();
        __syncthreads();
        if (ok) ok = mbar_wait(&wbar[buf], wph[buf], a.polls);
        ok = __syncthreads_and(ok);  // one verdict for the block
        if (ok) {  // the image landed
            wph[buf] ^= 1;
            pend[buf] = false;
            if (threadIdx.x == 0) {
                tc_fence_after();
                const uint32_t sbo = (uint32_t)(K / 8 * 128);
                const uint32_t idesc = tc_idesc_bf16(128, N);
                for (int kk = 0; kk < K / 16; kk++)
                    tc_mma_bf16(tbase + dcol, tc_desc(smem_u32(act) + kk * 256, 128, sbo),
                                tc_desc(smem_u32(wbuf[buf]) + kk * 256, 128, sbo), idesc, kk > 0);
                tc_commit(&bar);
                if (q + 1 < nimg) {  // the other buffer's last reader finished before this image began
                    const int nx = (q + 1) % WIMG_N;
                    mbar_expect_tx(&wbar[buf ^ 1], wimg_bytes(nx));
                    bulk_g2s(wbuf[buf ^ 1], a.img + wimg_off(nx), wimg_bytes(nx), &wbar[buf ^ 1]);
                }
            }
            if (q + 1 < nimg) pend[buf ^ 1] = true;
            ok = mbar_wait(&bar, phase, a.polls);
            ok = __syncthreads_and(ok);
            if (ok)
                phase ^= 1;
            else
                mpend = true;
        }
        q++;
        tc_fence_after();
    };
    auto hidden_epilogue = [&](int l) {
        // TMEM (256 columns) + bias, SiLU -> BF16 activations (K = 256 layout) in act
        const float* bl = bias + l * MLP_H;
        const int r = quarter * 32 + lane;
#pragma unroll 1
        for (int c = chalf * (MLP_H / 2); c < (chalf + 1) * (MLP_H / 2); c += 16) {
            float v[16];
            tmem_ld16(trow + c, v);
#pragma unroll
            for (int h = 0; h < 2; h++) {
                __align__(16) __nv_bfloat162 o[4];
#pragma unroll
                for (int j = 0; j < 4; j++)
                    o[j] = __floats2bfloat162_rn(silu_bf(v[h * 8 + 2 * j] + bl[c + h * 8 + 2 * j]),
                                                 silu_bf(v[h * 8 + 2 * j + 1] + bl[c + h * 8 + 2 * j + 1]));
                *reinterpret_cast<uint4*>(act + tc_off(r, c + h * 8, MLP_H)) = *reinterpret_cast<uint4*>(o);
            }
        }
        tc_fence_before();
    };
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int m0 = tile * 128;
        if (ok) {   // input: normalise, split into BF16 hi + lo, K = 128 layout (hi | lo)
            const int r = threadIdx.x & 127, row = m0 + r, k8h = (threadIdx.x >> 7) * 4;
#pragma unroll
            for (int k8 = k8h; k8 < k8h + 4; k8++) {
                __align__(16) __nv_bfloat16 hi[8], lo[8];
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    const int c = k8 * 8 + j;
                    const float x = row < a.B ? a.X[(size_t)row * MLP_IN + c] : 0.f;
                    const float xn = (x - nrm[c]) * nrm[MLP_IN + c];
                    hi[j] = __float2bfloat16(xn);
                    lo[j] = __float2bfloat16(xn - __bfloat162float(hi[j]));
                }
                *reinterpret_cast<uint4*>(act + tc_off(r, k8 * 8, MLP_K0)) = *reinterpret_cast<uint4*>(hi);
                *reinterpret_cast<uint4*>(act + tc_off(r, MLP_IN + k8 * 8, MLP_K0)) = *reinterpret_cast<uint4*>(lo);
            }
        }
        mma_img(0, MLP_K0, MLP_H);    // layer 0
        if (ok) hidden_epilogue(0);
        mma_img(0, MLP_H, 128);       // layer 1, outputs 0-127
        mma_img(128, MLP_H, 128);     //          outputs 128-255
        if (ok) hidden_epilogue(1);
        mma_img(0, MLP_H, 128);       // layer 2
        mma_img(128, MLP_H, 128);
        if (ok) hidden_epilogue(2);
        mma_img(0, MLP_H, MLP_OUT);   // layer 3
        if (ok) {   // output: + bias, de-normalise, threshold
            const int r = quarter * 32 + lane, row = m0 + r;
#pragma unroll 1
            for (int c = chalf * (MLP_OUT / 2); c < (chalf + 1) * (MLP_OUT / 2); c += 16) {
                float v[16];
                tmem_ld16(trow + c, v);
                if (row < a.B) {
#pragma unroll
                    for (int j = 0; j < 16; j++) {
                        const int cc = c + j;
                        const float z = v[j] + bias[3 * MLP_H + cc];
                        const float y = z * nrm[2 * MLP_IN + MLP_OUT + cc] + nrm[2 * MLP_IN + cc];
                        a.Y[(size_t)row * MLP_OUT + cc] =
                            cc < MLP_NY && fabsf(y) >= nrm[2 * MLP_IN + 2 * MLP_OUT + cc] ? y : 0.f;
                    }
                }
            }
            tc_fence_before();
        }
    }
    if (!ok) {
        // a wait gave up: give the copies and MMAs still in flight a last
        // bounded chance to finish before TMEM and shared memory are released
        if (pend[0]) mbar_wait(&wbar[0], wph[0], MB_POLLS);
        if (pend[1]) mbar_wait(&wbar[1], wph[1], MB_POLLS);
        if (mpend) mbar_wait(&bar, phase, MB_POLLS);
        if (threadIdx.x == 0) atomicAdd(a.err, 1u);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tbase, 256);
}

// ---------------------------------------------------------------------------
// training helpers
// ---------------------------------------------------------------------------
// normalised features as BF16 pairs: Xb[row] = (hi[0..63] | lo[0..63])
__global__ void k_prep_in(const float* X, const float* norm, __nv_bfloat16* Xb, int B) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B * MLP_IN) return;
    const int r = i / MLP_IN, c = i - r * MLP_IN;
    const float xn = (X[i] - norm[c]) / norm[MLP_IN + c];
    const __nv_bfloat16 hi = __float2bfloat16(xn);
    Xb[(size_t)r * MLP_K0 + c] = hi;
    Xb[(size_t)r * MLP_K0 + MLP_IN + c] = __float2bfloat16(xn - __bfloat162float(hi));
}

// gradient of W0 from that of [W0 | W0]: g[o][k] = gc[o][k] + gc[o][k + 64]
__global__ void k_fold_w0(const float* gc, float* g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= MLP_H * MLP_IN) return;
    const int o = i / MLP_IN, k = i - o * MLP_IN;
    g[i] = gc[(size_t)o * MLP_K0 + k] + gc[(size_t)o * MLP_K0 + MLP_IN + k];
}

// [W0 | W0] in BF16 (256 x 128)
__global__ void k_w0_pair(const __nv_bfloat16* W0, __nv_bfloat16* W0c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= MLP_H * MLP_K0) return;
    const int o = i / MLP_K0, k = i - o * MLP_K0;
    W0c[i] = W0[(size_t)o * MLP_IN + (k < MLP_IN ? k : k - MLP_IN)];
}

// loss of the normalised outputs (57 used columns); dZ = d loss / d Z in BF16
__global__ void k_loss(const float* Z, const float* Y, const float* norm, __nv_bfloat16* dZ, float* loss, int B) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float d2 = 0.f;
    if (i < B * MLP_OUT) {
        const int c = i % MLP_OUT;
        float g = 0.f;
        const float sd = norm[2 * MLP_IN + MLP_OUT + c];
        if (c < MLP_NY && sd > 0.f) {  // sd = 0: an output switched off (the plain start is kept)
            const float yn = (Y[i] - norm[2 * MLP_IN + c]) / sd;
            const float d = Z[i] - yn;
            d2 = d * d;
            g = 2.f * d / ((float)B * MLP_NY);
        }
        dZ[i] = __float2bfloat16(g);
    }
    for (int o = 16; o; o >>= 1) d2 += __shfl_xor_sync(0xffffffffu, d2, o);
    if ((threadIdx.x & 31) == 0 && d2 != 0.f) atomicAdd(loss, d2 / ((float)B * MLP_NY));
}

// dst[C x R] = src[R x C]^T (BF16), 32 x 32 tiles
__global__ void k_transpose_bf16(const __nv_bfloat16* src, __nv_bfloat16* dst, int R, int C) {
    __shared__ __nv_bfloat16 t[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int r = r0 + y, c = c0 + threadIdx.x;
        if (r < R && c < C) t[y][threadIdx.x] = src[(size_t)r * C + c];
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int c = c0 + y, r = r0 + threadIdx.x;
        if (r < R && c < C) dst[(size_t)c * R + r] = t[threadIdx.x][y];
    }
}

// out[n] = sum over rows of dZ[:, n]
__global__ void k_colsum(const __nv_bfloat16* dZ, float* out, int B, int N) {
    const int n = blockIdx.x;
    float s = 0.f;
    for (int r = threadIdx.x; r < B; r += blockDim.x) s += __bfloat162float(dZ[(size_t)r * N + n]);
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ float w[32];
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += w[i];
        out[n] = t;
    }
}

// Adam (Kingma & Ba 2015) on the FP32 master parameters
__global__ void k_adam(float* p, const float* g, float* m, float* v, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// BF16 copies of W (out x in) and W^T (in x out)
__global__ void k_wcast(const float* W, __nv_bfloat16* Wb, __nv_bfloat16* WTb, int out, int in) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= out * in) return;
    const int o = i / in, k = i - o * in;
    const __nv_bfloat16 v = __float2bfloat16(W[i]);
    Wb[i] = v;
    WTb[(size_t)k * out + o] = v;
}

}  // namespace rpb

using namespace rpb;

// ---------------------------------------------------------------------------
// test entry: C = A B^T on device arrays (M%128 == 0 not required; K%64 == 0,
// N%16 == 0, N <= 256 per tile column)
// ---------------------------------------------------------------------------
extern "C" int reprobus_tc_gemm_test(const void* A, const void* B, float* C, int M, int N, int K,
                                     unsigned int* err_dev, void* stream) {
    if (!A || !B || !C || !err_dev || M <= 0 || N <= 0 || K <= 0 || K % 64 || N % 16) return 1;
    GemmArgs g{};
    g.A = (const __nv_bfloat16*)A;
    g.B = (const __nv_bfloat16*)B;
    g.M = M;
    g.N = N;
    g.K = K;
    g.C = C;
    g.err = err_dev;
    constexpr int BN = 128;
    const size_t smem = 128 * 64 * 2 + BN * 64 * 2 + 96 * 1024;  // padding: at most 2 CTAs per SM (TMEM)
    cudaFuncSetAttribute(k_gemm_tn<EPI_F32, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid((M + 127) / 128, (N + BN - 1) / BN);
    k_gemm_tn<EPI_F32, BN><<<grid, 128, smem, (cudaStream_t)stream>>>(g);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// ---------------------------------------------------------------------------
// the network object of the C-ABI
// ---------------------------------------------------------------------------
#include <cstdio>
#include <cstring>
#include <new>
#include <random>

#include "../../include/reprobus_chem.h"
#include "mlp_net.h"

namespace {

#define MLP_TRY(x)                                                    \
    do {                                                              \
        cudaError_t e_ = (x);                                         \
        if (e_ != cudaSuccess) return rpb::mlp_fail(#x, e_, __LINE__); \
    } while (0)

}  // namespace

namespace rpb {

int mlp_fail(const char* what, cudaError_t e, int line) {
    reprobus_set_error(REPROBUS_ERR_CUDA, "%s: %s (mlp_kernels.cu:%d)", what, cudaGetErrorString(e), line);
    return REPROBUS_ERR_CUDA;
}

static size_t wsize(int l) { return (size_t)mlp_fan_in(l) * mlp_fan_out(l); }

struct MlpNet {
    int cap = 0;  // training batch capacity (rows)
    float* P = nullptr;       // FP32 master parameters, packed W0 b0 W1 b1 W2 b2 W3 b3
    float* G = nullptr;       // gradients, same packing
    float* Mo = nullptr;      // Adam first moment
    float* Vo = nullptr;      // Adam second moment
    __nv_bfloat16* Wb[MLP_NL] = {};
    __nv_bfloat16* WTb[MLP_NL] = {};
    __nv_bfloat16* W0c = nullptr;  // [W0 | W0] (256 x 128), the layer-0 operand for the hi/lo input pairs
    uint8_t* img = nullptr;        // weight images of the inference kernel
    float* Gc = nullptr;           // gradient of [W0 | W0]
    float* norm = nullptr;    // in_mean, in_std, out_mean, out_std
    int step = 0;
    int nsm = 0;  // SM count (set on the first inference)
    // training activations
    __nv_bfloat16* X = nullptr;
    float* Z[MLP_NL] = {};
    __nv_bfloat16* H[MLP_NL] = {};
    __nv_bfloat16* dZ[MLP_NL] = {};
    __nv_bfloat16* T1 = nullptr;  // transposes (cap x 256 each)
    __nv_bfloat16* T2 = nullptr;
    float* loss = nullptr;
    unsigned int* err = nullptr;
    uint32_t polls = MB_POLLS;  // inference wait limit (reprobus_mlp_set_wait_limit)
    float* W(int l) const {
        size_t o = 0;
        for (int i = 0; i < l; i++) o += wsize(i) + mlp_fan_out(i);
        return P + o;
    }
    size_t off(int l) const {
        size_t o = 0;
        for (int i = 0; i < l; i++) o += wsize(i) + mlp_fan_out(i);
        return o;
    }
};

static void free_net(MlpNet* n) {
    if (!n) return;
    cudaFree(n->P);
    cudaFree(n->G);
    cudaFree(n->Mo);
    cudaFree(n->Vo);
    for (int l = 0; l < MLP_NL; l++) {
        cudaFree(n->Wb[l]);
        cudaFree(n->WTb[l]);
        cudaFree(n->Z[l]);
        cudaFree(n->H[l]);
        cudaFree(n->dZ[l]);
    }
    cudaFree(n->W0c);
    cudaFree(n->img);
    cudaFree(n->Gc);
    cudaFree(n->norm);
    cudaFree(n->X);
    cudaFree(n->T1);
    cudaFree(n->T2);
    cudaFree(n->loss);
    cudaFree(n->err);
    delete n;
}

static int refresh_bf16(MlpNet* n, cudaStream_t s) {
    for (int l = 0; l < MLP_NL; l++) {
        const int out = mlp_fan_out(l), in = mlp_fan_in(l);
        k_wcast<<<(out * in + 255) / 256, 256, 0, s>>>(n->P + n->off(l), n->Wb[l], n->WTb[l], out, in);
    }
    k_w0_pair<<<(MLP_H * MLP_K0 + 255) / 256, 256, 0, s>>>(n->Wb[0], n->W0c);
    k_wimage<<<(WIMG_CHUNKS + 255) / 256, 256, 0, s>>>(n->W0c, n->Wb[1], n->Wb[2], n->Wb[3], n->img);
    MLP_TRY(cudaGetLastError());
    return REPROBUS_OK;
}

template <int EPI, int BN>
static int gemm(const GemmArgs& g, cudaStream_t s) {
    // shared memory sized so that at most 512 / BN blocks share an SM (their TMEM fits)
    const size_t need = 128 * 64 * 2 + BN * 64 * 2;
    const size_t per_sm = 227 * 1024;
    const int max_blocks = 512 / (BN < 32 ? 32 : BN);
    size_t smem = per_sm / max_blocks + 1024;
    if (smem < need) smem = need;
    if (smem > per_sm) smem = per_sm;
    MLP_TRY(cudaFuncSetAttribute(k_gemm_tn<EPI, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((g.M + 127) / 128, (g.N + BN - 1) / BN);
    k_gemm_tn<EPI, BN><<<grid, 128, smem, s>>>(g);
    MLP_TRY(cudaGetLastError());
    return REPROBUS_OK;
}

template <int EPI>
static int gemm_n(const GemmArgs& g, cudaStream_t s) {
    if (g.N <= 64) return gemm<EPI, 64>(g, s);
    if (g.N <= 128) return gemm<EPI, 128>(g, s);
    return gemm<EPI, 256>(g, s);
}

static int transpose(const __nv_bfloat16* src, __nv_bfloat16* dst, int R, int C, cudaStream_t s) {
    dim3 grid((C + 31) / 32, (R + 31) / 32);
    k_transpose_bf16<<<grid, dim3(32, 8), 0, s>>>(src, dst, R, C);
    MLP_TRY(cudaGetLastError());
    return REPROBUS_OK;
}

// forward + loss + backward of one batch into n->G; loss (mean squared error
// of the normalised outputs) accumulated in n->loss
static int forward_backward(MlpNet* n, const float* X, const float* Y, int B, cudaStream_t s) {
    int rc;
    MLP_TRY(cudaMemsetAsync(n->loss, 0, sizeof(float), s));
    k_prep_in<<<(B * MLP_IN + 255) / 256, 256, 0, s>>>(X, n->norm, n->X, B);
    for (int l = 0; l < MLP_NL; l++) {
        GemmArgs g{};
        g.A = l == 0 ? n->X : n->H[l - 1];
        g.B = l == 0 ? n->W0c : n->Wb[l];
        g.M = B;
        g.N = mlp_fan_out(l);
        g.K = l == 0 ? MLP_K0 : mlp_fan_in(l);
        g.C = n->Z[l];
        g.bias = n->P + n->off(l) + wsize(l);
        g.H = n->H[l];
        g.act = l < MLP_NL - 1;
        g.err = n->err;
        if ((rc = gemm_n<EPI_FWD>(g, s))) return rc;
    }
    k_loss<<<(B * MLP_OUT + 255) / 256, 256, 0, s>>>(n->Z[MLP_NL - 1], Y, n->norm, n->dZ[MLP_NL - 1], n->loss, B);
    for (int l = MLP_NL - 1; l >= 0; l--) {
        const int out = mlp_fan_out(l), in = mlp_fan_in(l);
        // dW = dZ^T A  (out x in), K = batch
        const int kin = l == 0 ? MLP_K0 : in;
        if ((rc = transpose(n->dZ[l], n->T1, B, out, s))) return rc;
        if ((rc = transpose(l == 0 ? n->X : n->H[l - 1], n->T2, B, kin, s))) return rc;
        GemmArgs g{};
        g.A = n->T1;
        g.B = n->T2;
        g.M = out;
        g.N = kin;
        g.K = B;
        g.C = l == 0 ? n->Gc : n->G + n->off(l);
        g.err = n->err;
        if ((rc = gemm_n<EPI_F32>(g, s))) return rc;
        if (l == 0) k_fold_w0<<<(MLP_H * MLP_IN + 255) / 256, 256, 0, s>>>(n->Gc, n->G);
        k_colsum<<<out, 256, 0, s>>>(n->dZ[l], n->G + n->off(l) + wsize(l), B, out);
        if (l > 0) {
            // dZ_{l-1} = (dZ_l W_l) * SiLU'(Z_{l-1})
            GemmArgs d{};
            d.A = n->dZ[l];
            d.B = n->WTb[l];
            d.M = B;
            d.N = in;
            d.K = out;
            d.H = n->dZ[l - 1];
            d.Zprev = n->Z[l - 1];
            d.err = n->err;
            if ((rc = gemm_n<EPI_BWD_SILU>(d, s))) return rc;
        }
    }
    MLP_TRY(cudaGetLastError());
    return REPROBUS_OK;
}

static int check_err(MlpNet* n, cudaStream_t s) {
    unsigned int e = 0;
    MLP_TRY(cudaMemcpyAsync(&e, n->err, sizeof(e), cudaMemcpyDeviceToHost, s));
    MLP_TRY(cudaStreamSynchronize(s));
    if (e) {
        reprobus_set_error(REPROBUS_ERR_TIMEOUT, "a tensor-core wait gave up (%u)", e);
        return REPROBUS_ERR_TIMEOUT;
    }
    return REPROBUS_OK;
}

int mlp_infer(void* net, const float* X, float* Y, int B, cudaStream_t s, const int* rows_dev) {
    MlpNet* n = (MlpNet*)net;
    InferArgs a{};
    a.X = X;
    a.Y = Y;
    a.B = B;
    a.Bdev = rows_dev;
    a.img = n->img;
    for (int l = 0; l < MLP_NL; l++) a.b[l] = n->P + n->off(l) + wsize(l);
    a.norm = n->norm;
    a.err = n->err;
    a.polls = n->polls;
    const size_t smem = 196608 + (3 * MLP_H + MLP_OUT + MLP_NNORM) * sizeof(float);
    if (!n->nsm) {  // once per network (not while a graph is being captured)
        int dev = 0;
        MLP_TRY(cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        MLP_TRY(cudaGetDevice(&dev));
        MLP_TRY(cudaDeviceGetAttribute(&n->nsm, cudaDevAttrMultiProcessorCount, dev));
    }
    const int nsm = n->nsm;
    const int tiles = (B + 127) / 128;
    k_mlp_infer<<<tiles < nsm ? tiles : nsm, MLP_INFER_THREADS, smem, s>>>(a);
    MLP_TRY(cudaGetLastError());
    return REPROBUS_OK;
}

unsigned int* mlp_err_flag(void* net) { return ((MlpNet*)net)->err; }

}  // namespace rpb

extern "C" int reprobus_mlp_create(int batch_cap, unsigned long long seed, void** out) {
    if (!out) return reprobus_set_error(REPROBUS_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (batch_cap <= 0 || batch_cap % 128)
        return reprobus_set_error(REPROBUS_ERR_ARG, "batch_cap must be a positive multiple of 128");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return reprobus_set_error(REPROBUS_ERR_NODEVICE, "no CUDA device visible");
    MlpNet* n = new (std::nothrow) MlpNet();
    if (!n) return reprobus_set_error(REPROBUS_ERR_ARG, "out of host memory");
    n->cap = batch_cap;
    auto fail = [&](int rc) {
        free_net(n);
        return rc;
    };
    const size_t np = MLP_NPARAM;
    cudaError_t e = cudaSuccess;
    auto al = [&](void** p, size_t b) {
        if (e == cudaSuccess) e = cudaMalloc(p, b);
    };
    al((void**)&n->P, np * 4);
    al((void**)&n->G, np * 4);
    al((void**)&n->Mo, np * 4);
    al((void**)&n->Vo, np * 4);
    for (int l = 0; l < MLP_NL; l++) {
        al((void**)&n->Wb[l], wsize(l) * 2);
        al((void**)&n->WTb[l], wsize(l) * 2);
        al((void**)&n->Z[l], (size_t)batch_cap * mlp_fan_out(l) * 4);
        al((void**)&n->H[l], (size_t)batch_cap * mlp_fan_out(l) * 2);
        al((void**)&n->dZ[l], (size_t)batch_cap * mlp_fan_out(l) * 2);
    }
    al((void**)&n->W0c, (size_t)MLP_H * MLP_K0 * 2);
    al((void**)&n->img, WIMG_TOTAL);
    al((void**)&n->Gc, (size_t)MLP_H * MLP_K0 * 4);
    al((void**)&n->norm, MLP_NNORM * 4);
    al((void**)&n->X, (size_t)batch_cap * MLP_K0 * 2);
    al((void**)&n->T1, (size_t)batch_cap * MLP_H * 2);
    al((void**)&n->T2, (size_t)batch_cap * MLP_H * 2);
    al((void**)&n->loss, 4);
    al((void**)&n->err, 4);
    if (e != cudaSuccess) return fail(reprobus_set_error(REPROBUS_ERR_CUDA, "mlp alloc: %s", cudaGetErrorString(e)));
    // initial parameters: uniform(-a, a), a = sqrt(6 / fan_in) (He), zero biases
    float* h = new (std::nothrow) float[np];
    if (!h) return fail(reprobus_set_error(REPROBUS_ERR_ARG, "out of host memory"));
    std::mt19937_64 rng(seed);
    size_t o = 0;
    for (int l = 0; l < MLP_NL; l++) {
        const float a = std::sqrt(6.f / mlp_fan_in(l)) * (l == MLP_NL - 1 ? 0.1f : 1.f);
        std::uniform_real_distribution<float> U(-a, a);
        for (size_t i = 0; i < wsize(l); i++) h[o++] = U(rng);
        for (int i = 0; i < mlp_fan_out(l); i++) h[o++] = 0.f;
    }
    float nrm[MLP_NNORM];
    for (int i = 0; i < MLP_IN; i++) {
        nrm[i] = 0.f;
        nrm[MLP_IN + i] = 1.f;
    }
    for (int i = 0; i < MLP_OUT; i++) {
        nrm[2 * MLP_IN + i] = 0.f;
        nrm[2 * MLP_IN + MLP_OUT + i] = 1.f;
        nrm[2 * MLP_IN + 2 * MLP_OUT + i] = 0.f;
    }
    if ((e = cudaMemcpy(n->P, h, np * 4, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(n->norm, nrm, sizeof(nrm), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemset(n->Mo, 0, np * 4)) != cudaSuccess || (e = cudaMemset(n->Vo, 0, np * 4)) != cudaSuccess ||
        (e = cudaMemset(n->err, 0, 4)) != cudaSuccess) {
        delete[] h;
        return fail(reprobus_set_error(REPROBUS_ERR_CUDA, "mlp init: %s", cudaGetErrorString(e)));
    }
    delete[] h;
    int rc = refresh_bf16(n, 0);
    if (rc) return fail(rc);
    if ((e = cudaDeviceSynchronize()) != cudaSuccess)
        return fail(reprobus_set_error(REPROBUS_ERR_CUDA, "mlp init: %s", cudaGetErrorString(e)));
    *out = n;
    return REPROBUS_OK;
}

extern "C" int reprobus_mlp_free(void* net) {
    free_net((MlpNet*)net);
    return REPROBUS_OK;
}

extern "C" int reprobus_mlp_nparams(void) { return MLP_NPARAM; }

extern "C" int reprobus_mlp_set_params(void* net, const float* params, const float* norm) {
    MlpNet* n = (MlpNet*)net;
    if (!n) return reprobus_set_error(REPROBUS_ERR_ARG, "net is NULL");
    if (params) MLP_TRY(cudaMemcpy(n->P, params, (size_t)MLP_NPARAM * 4, cudaMemcpyHostToDevice));
    if (norm) MLP_TRY(cudaMemcpy(n->norm, norm, MLP_NNORM * 4, cudaMemcpyHostToDevice));
    int rc = refresh_bf16(n, 0);
    if (rc) return rc;
    MLP_TRY(cudaDeviceSynchronize());
    return REPROBUS_OK;
}

extern "C" int reprobus_mlp_get_params(void* net, float* params, float* norm) {
    MlpNet* n = (MlpNet*)net;
    if (!n) return reprobus_set_error(REPROBUS_ERR_ARG, "net is NULL");
    MLP_TRY(cudaDeviceSynchronize());
    if (params) MLP_TRY(cudaMemcpy(params, n->P, (size_t)MLP_NPARAM * 4, cudaMemcpyDeviceToHost));
    if (norm) MLP_TRY(cudaMemcpy(norm, n->norm, MLP_NNORM * 4, cudaMemcpyDeviceToHost));
    return REPROBUS_OK;
}

static int check_batch(MlpNet* n, const float* X, const float* Y, int B) {
    if (!n) return reprobus_set_error(REPROBUS_ERR_ARG, "net is NULL");
    if (!X || !Y) return reprobus_set_error(REPROBUS_ERR_ARG, "X and Y must be device pointers");
    if (B <= 0 || B > n->cap || B % 128)
        return reprobus_set_error(REPROBUS_ERR_ARG, "batch %d: a multiple of 128 up to %d", B, n->cap);
    return REPROBUS_OK;
}

extern "C" int reprobus_mlp_grads(void* net, const float* X, const float* Y, int B, float* grads, float* loss,
                                  void* stream) {
    MlpNet* n = (MlpNet*)net;
    int rc = check_batch(n, X, Y, B);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if ((rc = forward_backward(n, X, Y, B, s))) return rc;
    if ((rc = check_err(n, s))) return rc;
    if (grads) MLP_TRY(cudaMemcpy(grads, n->G, (size_t)MLP_NPARAM * 4, cudaMemcpyDeviceToHost));
    if (loss) MLP_TRY(cudaMemcpy(loss, n->loss, 4, cudaMemcpyDeviceToHost));
    return REPROBUS_OK;
}

extern "C" int reprobus_mlp_train_step(void* net, const float* X, const float* Y, int B, float lr, float* loss,
                                       void* stream) {
    MlpNet* n = (MlpNet*)net;
    int rc = check_batch(n, X, Y, B);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if ((rc = forward_backward(n, X, Y, B, s))) return rc;
    n->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)n->step), c2 = 1.f - std::pow(b2, (float)n->step);
    k_adam<<<(MLP_NPARAM + 255) / 256, 256, 0, s>>>(n->P, n->G, n->Mo, n->Vo, MLP_NPARAM, lr, b1, b2, 1e-8f, c1, c2);
    MLP_TRY(cudaGetLastError());
    if ((rc = refresh_bf16(n, s))) return rc;
    if (loss) {
        MLP_TRY(cudaMemcpyAsync(loss, n->loss, 4, cudaMemcpyDeviceToHost, s));
        if ((rc = check_err(n, s))) return rc;
    }
    return REPROBUS_OK;
}

extern "C" int reprobus_mlp_forward(void* net, const float* X, float* Y, int B, void* stream) {
    MlpNet* n = (MlpNet*)net;
    if (!n) return reprobus_set_error(REPROBUS_ERR_ARG, "net is NULL");
    if (!X || !Y || B <= 0) return reprobus_set_error(REPROBUS_ERR_ARG, "bad forward arguments");
    cudaStream_t s = (cudaStream_t)stream;
    MLP_TRY(cudaMemsetAsync(n->err, 0, sizeof(unsigned int), s));
    int rc = mlp_infer(n, X, Y, B, s);
    if (rc) return rc;
    return check_err(n, s);
}

extern "C" int reprobus_mlp_set_wait_limit(void* net, long long polls) {
    MlpNet* n = (MlpNet*)net;
    if (!n) return reprobus_set_error(REPROBUS_ERR_ARG, "net is NULL");
    if (polls > 0xffffffffLL) return reprobus_set_error(REPROBUS_ERR_ARG, "polls above 2^32 - 1");
    n->polls = polls < 0 ? MB_POLLS : (uint32_t)polls;
    return REPROBUS_OK;
}
