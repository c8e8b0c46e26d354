// Chemistry surrogate network on the 5th-generation tensor cores: BF16 weights
// and activations, FP32 accumulation in tensor memory (tcgen05.mma, TMEM),
// operands staged in shared memory (tcgen05.cuh for the layouts).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "level.h"
#include "mlp_kernel.cuh"

namespace ocfd {

using namespace tc;

// C[128 x N] = A[128 x K] * B[N x K]^T for row-major BF16 A, B (K contiguous) and
// row-major FP32 C: one CTA of 128 threads, the whole K staged in shared memory.
__global__ void __launch_bounds__(128) k_tc_gemm(const uint16_t* __restrict__ A, const uint16_t* __restrict__ B,
                                                 float* __restrict__ C, int N, int K, unsigned* err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char* sA = sm;
    unsigned char* sB = sm + 128 * K * 2;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sB + N * K * 2);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t ncols = tmem_cols(N);
    for (int e = tid; e < 128 * K; e += 128)
        *reinterpret_cast<uint16_t*>(sA + kmajor_offset(e / K, e % K, 128)) = A[e];
    for (int e = tid; e < N * K; e += 128)
        *reinterpret_cast<uint16_t*>(sB + kmajor_offset(e / K, e % K, N)) = B[e];
    if (tid == 0) mbar_init(bar, 1);
    if (warp == 0) {
        tmem_alloc(tslot, ncols);
        tmem_relinquish();
    }
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tbase = *tslot;
    if (tid == 0) {
        const uint32_t idesc = idesc_bf16_f32(128, N);
        for (int ks = 0; ks < K / 16; ++ks)
            mma_bf16(tbase, smem_desc(smem_u32(sA + ks * 128 * 32)), smem_desc(smem_u32(sB + ks * N * 32)), idesc,
                     ks > 0 ? 1u : 0u);
        mma_commit(bar);
    }
    const bool ok = mbar_wait(bar, 0);
    fence_after_sync();
    if (!ok) {
        if (tid == 0) atomicOr(err, 1u);
    } else {
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tmem_ld16(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) C[(long long)tid * N + c0 + i] = v[i];
        }
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tbase, ncols);
}

// Training forward: X [M x 16] BF16 normalised inputs (row-major) -> Y [M x 16]
// FP32, stashing Z_l, H_l (l = 1..4) as [4][M/128][128 x 128] blocks; MLP_G
// warpgroups per 128-row tile (the first stages the inputs and writes Y).
__global__ void __launch_bounds__(128 * MLP_G) k_mlp_forward(MlpNet net, const uint16_t* __restrict__ X, float* Y,
                                                             float* Z, uint16_t* H, int ntile, unsigned* err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + S_BAR);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + S_BAR + 8);
    const int tid = threadIdx.x, warp = tid >> 5;
    mlp_stage_weights(net, sm);
    if (tid == 0) mbar_init(bar, 1);
    if (warp == 0) {
        tmem_alloc(tslot, 128);
        tmem_relinquish();
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tbase = *tslot;
    uint32_t phase = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < ntile && ok; t += gridDim.x) {
        const long long row = (long long)t * 128 + tid;
        if (tid < 128) {
            // one row of 16 BF16 inputs: two 16-byte core-matrix rows
            const uint4* xr = reinterpret_cast<const uint4*>(X + row * 16);
            *reinterpret_cast<uint4*>(sm + S_A0 + kmajor_offset(tid, 0, 128)) = xr[0];
            *reinterpret_cast<uint4*>(sm + S_A0 + kmajor_offset(tid, 8, 128)) = xr[1];
        }
        float out[16];
        // stash layout: block t of layer l at ((l * ntile + t) * 128 + row) * 128
        ok = mlp_tile<MLP_G>(sm, tbase, bar, phase, out, Z ? Z + (long long)t * 128 * 128 : nullptr,
                             H ? H + (long long)t * 128 * 128 : nullptr, (long long)ntile * 128);
        if (ok && tid < 128)
#pragma unroll
            for (int i = 0; i < 16; ++i) Y[row * 16 + i] = out[i];
    }
    if (!ok && tid == 0) atomicOr(err, 1u);
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tbase, 128);
}

__device__ __forceinline__ float gelu_grad(float z) {
    return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// pack normalised FP32 features [M x 12] into the BF16 input operand rows [M x 16]
__global__ void k_mlp_pack(const float* __restrict__ X, uint16_t* Xb, long long M) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < M * 16;
         e += (long long)gridDim.x * blockDim.x) {
        const long long m = e >> 4;
        const int k = (int)(e & 15);
        Xb[e] = k < MLP_IN ? bf16_bits(X[m * MLP_IN + k]) : (uint16_t)0;
    }
}

// loss = mean over rows and the 10 outputs of (Y - T)^2; dY = dloss / dY into
// dZ4 [M x 16] (zero on the padding); per-block partial sums of the loss
__global__ void k_mlp_out_grad(const float* __restrict__ Y, const float* __restrict__ T, float* dZ4, long long M,
                               float* lossp) {
    __shared__ float red[256];
    float acc = 0.0f;
    const float scale = 2.0f / (float)(M * MLP_OUT);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < M * 16;
         e += (long long)gridDim.x * blockDim.x) {
        const long long m = e >> 4;
        const int j = (int)(e & 15);
        float g = 0.0f;
        if (j < MLP_OUT) {
            const float d = Y[e] - T[m * MLP_OUT + j];
            acc += d * d;
            g = scale * d;
        }
        dZ4[e] = g;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) lossp[blockIdx.x] = red[0];
}

// dZ_{l-1} = (dZ_l W_l) * gelu'(Z_{l-1}) for layer l = 1..4, 128-row tiles:
// A = dZ_l (128 x N_l, BF16), B(j, n) = W_l[n][j] (K_l x N_l), D = 128 x 128
constexpr int SD_A = 0, SD_B = 128 * 128 * 2, SD_BAR = 2 * 128 * 128 * 2, SD_TOT = SD_BAR + 16;

__global__ void __launch_bounds__(128) k_mlp_bwd_data(MlpNet net, int l, const float* __restrict__ dZl,
                                                      const float* __restrict__ Zprev, float* dZprev, int ntile,
                                                      unsigned* err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + SD_BAR);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + SD_BAR + 8);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int N = LN(l), K = LK(l);  // this layer: N outputs, K inputs (= 128)
    for (int e = tid; e < N * K; e += 128) {
        const int n = e / K, j = e % K;
        *reinterpret_cast<uint16_t*>(sm + SD_B + kmajor_offset(j, n, K)) = net.W[WOFF(l) + e];
    }
    if (tid == 0) mbar_init(bar, 1);
    if (warp == 0) {
        tmem_alloc(tslot, 128);
        tmem_relinquish();
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tbase = *tslot;
    const uint32_t trow = tbase + ((uint32_t)(warp * 32) << 16);
    uint32_t phase = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < ntile && ok; t += gridDim.x) {
        const long long row = (long long)t * 128 + tid;
        for (int n = 0; n < N; ++n)
            *reinterpret_cast<uint16_t*>(sm + SD_A + kmajor_offset(tid, n, 128)) = bf16_bits(dZl[row * N + n]);
        fence_async_smem();
        fence_before_sync();
        __syncthreads();
        fence_after_sync();
        if (tid == 0) {
            const uint32_t idesc = idesc_bf16_f32(128, K);
            for (int ks = 0; ks < N / 16; ++ks)
                mma_bf16(tbase, smem_desc(smem_u32(sm + SD_A + ks * 128 * 32)),
                         smem_desc(smem_u32(sm + SD_B + ks * K * 32)), idesc, ks > 0 ? 1u : 0u);
            mma_commit(bar);
        }
        ok = mbar_wait(bar, phase);
        phase ^= 1u;
        fence_after_sync();
        if (!ok) break;
        for (int c0 = 0; c0 < 128; c0 += 32) {
            float v[32];
            tmem_ld32(trow + (uint32_t)c0, v);
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                const long long q = row * 128 + c0 + i;
                dZprev[q] = v[i] * gelu_grad(Zprev[q]);
            }
        }
        fence_before_sync();
        __syncthreads();
    }
    if (!ok && tid == 0) atomicOr(err, 1u);
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tbase, 128);
}

// Weight and bias gradients of layer l over one chunk of 256 rows (block c):
// dW_l[n][k] = sum_m dZ_l[m][n] A_l[m][k], db_l[n] = sum_m dZ_l[m][n], as
// partials partW[c][.], partb[c][.].  The tensor-core M dimension (128 rows)
// is n for l < 4 and k for l = 4 (whose N_l = 16); the MMA K dimension is the
// chunk's rows.
constexpr int CHUNK = 256;
constexpr int SW_A = 0, SW_B = 128 * CHUNK * 2, SW_BAR = 2 * 128 * CHUNK * 2, SW_TOT = SW_BAR + 16;

__global__ void __launch_bounds__(128) k_mlp_bwd_weight(int l, const float* __restrict__ dZl,
                                                        const uint16_t* __restrict__ Al, int lda, float* partW,
                                                        float* partb, unsigned* err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + SW_BAR);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + SW_BAR + 8);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int N = LN(l), K = LK(l);
    const long long m0 = (long long)blockIdx.x * CHUNK;
    const bool swap = (l == 4);
    const int ncol = swap ? N : K;  // columns of D
    // A: 128 rows (n, or k when swapped) x CHUNK; B: ncol rows x CHUNK
    for (int e = tid; e < 128 * CHUNK; e += 128) {
        const int r = e / CHUNK, mm = e % CHUNK;
        const long long m = m0 + mm;
        const uint16_t v = swap ? Al[m * lda + r] : bf16_bits(dZl[m * N + r]);
        *reinterpret_cast<uint16_t*>(sm + SW_A + kmajor_offset(r, mm, 128)) = v;
    }
    for (int e = tid; e < ncol * CHUNK; e += 128) {
        const int r = e / CHUNK, mm = e % CHUNK;
        const long long m = m0 + mm;
        const uint16_t v = swap ? bf16_bits(dZl[m * N + r]) : Al[m * lda + r];
        *reinterpret_cast<uint16_t*>(sm + SW_B + kmajor_offset(r, mm, ncol)) = v;
    }
    if (tid == 0) mbar_init(bar, 1);
    if (warp == 0) {
        tmem_alloc(tslot, 128);
        tmem_relinquish();
    }
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tbase = *tslot;
    if (tid == 0) {
        const uint32_t idesc = idesc_bf16_f32(128, ncol);
        for (int ks = 0; ks < CHUNK / 16; ++ks)
            mma_bf16(tbase, smem_desc(smem_u32(sm + SW_A + ks * 128 * 32)),
                     smem_desc(smem_u32(sm + SW_B + ks * ncol * 32)), idesc, ks > 0 ? 1u : 0u);
        mma_commit(bar);
    }
    // bias partial while the tensor core works: rows of the chunk in order
    if (tid < N) {
        float acc = 0.0f;
        for (int mm = 0; mm < CHUNK; ++mm) acc += dZl[(m0 + mm) * N + tid];
        partb[(long long)blockIdx.x * BTOT + BOFF(l) + tid] = acc;
    }
    const bool ok = mbar_wait(bar, 0);
    fence_after_sync();
    if (!ok) {
        if (tid == 0) atomicOr(err, 1u);
    } else {
        float* pw = partW + (long long)blockIdx.x * WTOT + WOFF(l);
        for (int c0 = 0; c0 < ncol; c0 += 16) {
            float v[16];
            tmem_ld16(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                // row tid, column c0 + i of D
                if (swap) pw[(c0 + i) * K + tid] = v[i];   // D[k][n] -> W[n][k]
                else pw[tid * K + c0 + i] = v[i];          // D[n][k]
            }
        }
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tbase, 128);
}

// gradients = sum of the chunk partials in chunk order; Adam step on the FP32
// master parameters (bias-corrected, Kingma & Ba 2015); BF16 copy of the weights
__global__ void k_mlp_reduce_adam(const float* __restrict__ partW, const float* __restrict__ partb, int nchunk,
                                  float* W32, float* b32, float* mW, float* vW, float* mb, float* vb, uint16_t* Wb,
                                  float* gW, float* gb, float lr, float c1, float c2, int update) {
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < WTOT + BTOT; i += gridDim.x * blockDim.x) {
        const bool isw = i < WTOT;
        const int q = isw ? i : i - WTOT;
        const float* part = isw ? partW : partb;
        const int stride = isw ? WTOT : BTOT;
        float g = 0.0f;
        for (int c = 0; c < nchunk; ++c) g += part[(long long)c * stride + q];
        if (gW && isw) gW[q] = g;
        if (gb && !isw) gb[q] = g;
        if (!update) continue;
        float* p = isw ? W32 + q : b32 + q;
        float* m = isw ? mW + q : mb + q;
        float* v = isw ? vW + q : vb + q;
        *m = beta1 * *m + (1.0f - beta1) * g;
        *v = beta2 * *v + (1.0f - beta2) * g * g;
        *p -= lr * (*m * c1) / (sqrtf(*v * c2) + eps);
        if (isw) Wb[q] = bf16_bits(*p);
    }
}

__global__ void k_mlp_to_bf16(const float* W32, uint16_t* Wb) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < WTOT; i += gridDim.x * blockDim.x)
        Wb[i] = bf16_bits(W32[i]);
}

}  // namespace ocfd

// ------------------------------------------------------------------ the object
struct ocfd_mlp {
    ocfd_context* ctx = nullptr;
    int max_batch = 0;
    float *W32 = nullptr, *b32 = nullptr, *mW = nullptr, *vW = nullptr, *mb = nullptr, *vb = nullptr;
    uint16_t* Wb = nullptr;
    float norm[2 * ocfd::MLP_IN + 3 * ocfd::MLP_OUT] = {};
    long long steps = 0;
    // training scratch (max_batch rows)
    uint16_t* Xb = nullptr;
    float* Y = nullptr;
    float* Z = nullptr;      // 4 x M x 128
    uint16_t* H = nullptr;   // 4 x M x 128
    float* dZ4 = nullptr;    // M x 16
    float* dZa = nullptr;    // M x 128
    float* dZb = nullptr;    // M x 128
    float* partW = nullptr;  // nchunk x WTOT
    float* partb = nullptr;  // nchunk x BTOT
    float* lossp = nullptr;
    float* gW = nullptr;
    float* gb = nullptr;
};

namespace ocfd {

MlpNet mlp_net(const ocfd_mlp* n);
static MlpNet net_of(const ocfd_mlp* n) { return mlp_net(n); }
MlpNet mlp_net(const ocfd_mlp* n) {
    MlpNet d{};
    d.W = n->Wb;
    d.b = n->b32;
    for (int i = 0; i < MLP_IN; ++i) {
        d.in_mu[i] = n->norm[i];
        d.in_isd[i] = n->norm[MLP_IN + i];
    }
    for (int i = 0; i < MLP_OUT; ++i) {
        d.out_mu[i] = n->norm[2 * MLP_IN + i];
        d.out_sd[i] = n->norm[2 * MLP_IN + MLP_OUT + i];
        d.out_scale[i] = n->norm[2 * MLP_IN + 2 * MLP_OUT + i];
    }
    return d;
}

static ocfd_status mlp_configure() {
    static bool done = false;
    if (done) return OCFD_OK;
    if (cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, S_TOT) != cudaSuccess ||
        cudaFuncSetAttribute(k_mlp_bwd_data, cudaFuncAttributeMaxDynamicSharedMemorySize, SD_TOT) != cudaSuccess ||
        cudaFuncSetAttribute(k_mlp_bwd_weight, cudaFuncAttributeMaxDynamicSharedMemorySize, SW_TOT) != cudaSuccess)
        return check_launch("MLP kernel attributes");
    done = true;
    return OCFD_OK;
}

// forward (+ stash) over M rows of normalised FP32 features
static ocfd_status mlp_forward(ocfd_mlp* n, const float* X, long long M, cudaStream_t st) {
    const int sms = n->ctx->num_sms;
    k_mlp_pack<<<grid_for(M * 16, 256, sms), 256, 0, st>>>(X, n->Xb, M);
    const int ntile = (int)(M / 128);
    k_mlp_forward<<<std::min(ntile, sms), 128 * MLP_G, S_TOT, st>>>(net_of(n), n->Xb, n->Y, n->Z, n->H, ntile,
                                                                    n->ctx->d_error);
    return check_launch("MLP forward");
}

static ocfd_status mlp_backward(ocfd_mlp* n, const float* T, long long M, cudaStream_t st, int nblk_loss) {
    const int sms = n->ctx->num_sms;
    const int ntile = (int)(M / 128), nchunk = (int)(M / CHUNK);
    k_mlp_out_grad<<<nblk_loss, 256, 0, st>>>(n->Y, T, n->dZ4, M, n->lossp);
    const MlpNet net = net_of(n);
    // layer 4 (output): weights from dZ4 and H4
    k_mlp_bwd_weight<<<nchunk, 128, SW_TOT, st>>>(4, n->dZ4, n->H + 3LL * M * 128, 128, n->partW, n->partb,
                                                   n->ctx->d_error);
    // dZ3 = (dZ4 W5) * gelu'(Z4)
    const float* dcur = n->dZ4;
    float* dnext = n->dZa;
    for (int l = 4; l >= 1; --l) {
        k_mlp_bwd_data<<<std::min(ntile, sms), 128, SD_TOT, st>>>(net, l, dcur, n->Z + (long long)(l - 1) * M * 128,
                                                                  dnext, ntile, n->ctx->d_error);
        // weights of layer l-1 from dZ_{l-1} and its input (H_{l-1}, or X for l-1 = 0)
        const uint16_t* A = (l - 1 == 0) ? n->Xb : n->H + (long long)(l - 2) * M * 128;
        k_mlp_bwd_weight<<<nchunk, 128, SW_TOT, st>>>(l - 1, dnext, A, (l - 1 == 0) ? 16 : 128, n->partW, n->partb,
                                                       n->ctx->d_error);
        dcur = dnext;
        dnext = (dnext == n->dZa) ? n->dZb : n->dZa;
    }
    (void)sms;
    return check_launch("MLP backward");
}

}  // namespace ocfd

using namespace ocfd;

extern "C" {

ocfd_status ocfd_mlp_create(ocfd_context* ctx, int32_t max_batch, uint64_t seed, ocfd_mlp** out) {
    if (!ctx || !out || max_batch < CHUNK || max_batch % CHUNK)
        return fail(OCFD_BAD_ARG, "ocfd_mlp_create: max_batch must be a positive multiple of 256");
    *out = nullptr;
    ocfd_status s = mlp_configure();
    if (s != OCFD_OK) return s;
    ocfd_mlp* n = new ocfd_mlp();
    n->ctx = ctx;
    n->max_batch = max_batch;
    const long long M = max_batch, nchunk = M / CHUNK;
    bool ok = true;
    auto al = [&](void** p, size_t bytes) {
        if (cudaMalloc(p, bytes) != cudaSuccess) ok = false;
        else cudaMemset(*p, 0, bytes);
    };
    al((void**)&n->W32, 4 * WTOT);
    al((void**)&n->b32, 4 * BTOT);
    al((void**)&n->mW, 4 * WTOT);
    al((void**)&n->vW, 4 * WTOT);
    al((void**)&n->mb, 4 * BTOT);
    al((void**)&n->vb, 4 * BTOT);
    al((void**)&n->Wb, 2 * WTOT);
    al((void**)&n->Xb, 2 * M * 16);
    al((void**)&n->Y, 4 * M * 16);
    al((void**)&n->Z, 4 * 4 * M * 128);
    al((void**)&n->H, 2 * 4 * M * 128);
    al((void**)&n->dZ4, 4 * M * 16);
    al((void**)&n->dZa, 4 * M * 128);
    al((void**)&n->dZb, 4 * M * 128);
    al((void**)&n->partW, 4 * nchunk * WTOT);
    al((void**)&n->partb, 4 * nchunk * BTOT);
    al((void**)&n->lossp, 4 * 1024);
    al((void**)&n->gW, 4 * WTOT);
    al((void**)&n->gb, 4 * BTOT);
    if (!ok) {
        cudaGetLastError();
        ocfd_mlp_destroy(n);
        return fail(OCFD_OUT_OF_MEMORY, "ocfd_mlp_create");
    }
    // He-normal initial weights (Box-Muller on a 64-bit LCG), zero biases and padding
    std::vector<float> W(WTOT, 0.0f);
    uint64_t x = seed * 6364136223846793005ull + 1442695040888963407ull;
    auto uni = [&]() {
        x = x * 6364136223846793005ull + 1442695040888963407ull;
        return ((x >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < 5; ++l) {
        const int N = LN(l), K = LK(l);
        const int kin = (l == 0) ? MLP_IN : K, nout = (l == 4) ? MLP_OUT : N;
        const double sd = std::sqrt(2.0 / kin);
        for (int i = 0; i < nout; ++i)
            for (int j = 0; j < kin; ++j) {
                const double u1 = uni(), u2 = uni();
                W[WOFF(l) + i * K + j] = (float)(sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
            }
    }
    for (int i = 0; i < MLP_IN; ++i) n->norm[MLP_IN + i] = 1.0f;
    for (int i = 0; i < MLP_OUT; ++i) n->norm[2 * MLP_IN + MLP_OUT + i] = 1.0f;
    cudaMemcpy(n->W32, W.data(), 4 * WTOT, cudaMemcpyHostToDevice);
    k_mlp_to_bf16<<<64, 256>>>(n->W32, n->Wb);
    s = check_launch("ocfd_mlp_create");
    if (s == OCFD_OK && cudaDeviceSynchronize() != cudaSuccess) s = check_launch("ocfd_mlp_create");
    if (s != OCFD_OK) {
        ocfd_mlp_destroy(n);
        return s;
    }
    *out = n;
    return OCFD_OK;
}

ocfd_status ocfd_mlp_destroy(ocfd_mlp* n) {
    if (!n) return OCFD_OK;
    void* ps[] = {n->W32, n->b32, n->mW, n->vW, n->mb, n->vb, n->Wb, n->Xb, n->Y, n->Z, n->H, n->dZ4, n->dZa,
                  n->dZb, n->partW, n->partb, n->lossp, n->gW, n->gb};
    for (void* p : ps) cudaFree(p);
    delete n;
    return OCFD_OK;
}

ocfd_status ocfd_mlp_set_norm(ocfd_mlp* n, const float* in_mu, const float* in_isd, const float* out_mu,
                              const float* out_sd) {
    if (!n || !in_mu || !in_isd || !out_mu || !out_sd) return fail(OCFD_BAD_ARG, "ocfd_mlp_set_norm");
    for (int i = 0; i < MLP_IN; ++i) {
        n->norm[i] = in_mu[i];
        n->norm[MLP_IN + i] = in_isd[i];
    }
    for (int i = 0; i < MLP_OUT; ++i) {
        n->norm[2 * MLP_IN + i] = out_mu[i];
        n->norm[2 * MLP_IN + MLP_OUT + i] = out_sd[i];
    }
    return OCFD_OK;
}

ocfd_status ocfd_mlp_set_target_scale(ocfd_mlp* n, const float* scale) {
    if (!n || !scale) return fail(OCFD_BAD_ARG, "ocfd_mlp_set_target_scale");
    for (int i = 0; i < MLP_OUT; ++i) n->norm[2 * MLP_IN + 2 * MLP_OUT + i] = scale[i];
    return OCFD_OK;
}

ocfd_status ocfd_mlp_get_params(ocfd_mlp* n, float* W, float* b) {
    if (!n) return fail(OCFD_BAD_ARG, "ocfd_mlp_get_params");
    if ((W && cudaMemcpy(W, n->W32, 4 * WTOT, cudaMemcpyDeviceToHost) != cudaSuccess) ||
        (b && cudaMemcpy(b, n->b32, 4 * BTOT, cudaMemcpyDeviceToHost) != cudaSuccess))
        return check_launch("ocfd_mlp_get_params");
    return OCFD_OK;
}

ocfd_status ocfd_mlp_set_params(ocfd_mlp* n, const float* W, const float* b) {
    if (!n) return fail(OCFD_BAD_ARG, "ocfd_mlp_set_params");
    if ((W && cudaMemcpy(n->W32, W, 4 * WTOT, cudaMemcpyHostToDevice) != cudaSuccess) ||
        (b && cudaMemcpy(n->b32, b, 4 * BTOT, cudaMemcpyHostToDevice) != cudaSuccess))
        return check_launch("ocfd_mlp_set_params");
    k_mlp_to_bf16<<<64, 256>>>(n->W32, n->Wb);
    return check_launch("ocfd_mlp_set_params");
}

static ocfd_status mlp_check_error(ocfd_mlp* n, cudaStream_t st, const char* who) {
    uint32_t e = 0;
    if (cudaMemcpyAsync(&e, n->ctx->d_error, sizeof(e), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return check_launch(who);
    if (e) {
        cudaMemsetAsync(n->ctx->d_error, 0, sizeof(uint32_t), st);
        return fail(OCFD_TIMEOUT, std::string(who) + ": a tensor-core completion wait ran out");
    }
    return OCFD_OK;
}

// Y [M x 10] = network(X [M x 12]) in normalised units (device arrays)
ocfd_status ocfd_mlp_forward(ocfd_mlp* n, const float* X, float* Y, int64_t M, void* stream) {
    if (!n || !X || !Y || M <= 0 || M % 128 || M > n->max_batch) return fail(OCFD_BAD_ARG, "ocfd_mlp_forward: M");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    ocfd_status s = mlp_forward(n, X, M, st);
    if (s != OCFD_OK) return s;
    if (cudaMemcpy2DAsync(Y, sizeof(float) * MLP_OUT, n->Y, sizeof(float) * 16, sizeof(float) * MLP_OUT, (size_t)M,
                          cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return check_launch("ocfd_mlp_forward");
    return mlp_check_error(n, st, "ocfd_mlp_forward");
}

// One training step on (X [M x 12], T [M x 10]) normalised device arrays:
// forward, MSE loss, backward, Adam (lr).  update = 0 computes the gradients
// only (gW [WTOT], gb [BTOT] on the host when given).  loss: host scalar.
ocfd_status ocfd_mlp_train_step(ocfd_mlp* n, const float* X, const float* T, int64_t M, float lr, int32_t update,
                                float* loss, float* gW, float* gb, void* stream) {
    if (!n || !X || !T || M <= 0 || M % CHUNK || M > n->max_batch)
        return fail(OCFD_BAD_ARG, "ocfd_mlp_train_step: M must be a multiple of 256 up to max_batch");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    ocfd_status s = mlp_forward(n, X, M, st);
    if (s != OCFD_OK) return s;
    const int nblk = 256;
    s = mlp_backward(n, T, M, st, nblk);
    if (s != OCFD_OK) return s;
    if (update) ++n->steps;
    const float c1 = update ? (float)(1.0 / (1.0 - std::pow(0.9, (double)n->steps))) : 1.0f;
    const float c2 = update ? (float)(1.0 / (1.0 - std::pow(0.999, (double)n->steps))) : 1.0f;
    k_mlp_reduce_adam<<<grid_for(WTOT + BTOT, 256, n->ctx->num_sms), 256, 0, st>>>(
        n->partW, n->partb, (int)(M / CHUNK), n->W32, n->b32, n->mW, n->vW, n->mb, n->vb, n->Wb, n->gW, n->gb, lr, c1,
        c2, update);
    s = check_launch("ocfd_mlp_train_step");
    if (s != OCFD_OK) return s;
    if (loss) {
        float lp[nblk];
        if (cudaMemcpyAsync(lp, n->lossp, sizeof(lp), cudaMemcpyDeviceToHost, st) != cudaSuccess)
            return check_launch("ocfd_mlp_train_step");
        s = mlp_check_error(n, st, "ocfd_mlp_train_step");
        if (s != OCFD_OK) return s;
        double acc = 0;
        for (int i = 0; i < nblk; ++i) acc += lp[i];
        *loss = (float)(acc / ((double)M * MLP_OUT));
    }
    if (gW && cudaMemcpyAsync(gW, n->gW, 4 * WTOT, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return check_launch("ocfd_mlp_train_step");
    if (gb && cudaMemcpyAsync(gb, n->gb, 4 * BTOT, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return check_launch("ocfd_mlp_train_step");
    return mlp_check_error(n, st, "ocfd_mlp_train_step");
}

}  // extern "C"

extern "C" ocfd_status ocfd_tc_gemm_bf16(ocfd_context* ctx, const uint16_t* A, const uint16_t* B, float* C, int N,
                                         int K, void* stream) {
    if (!ctx || !A || !B || !C || N < 16 || N > 256 || N % 16 || K < 16 || K > 256 || K % 16)
        return fail(OCFD_BAD_ARG, "ocfd_tc_gemm_bf16: N in [16, 256] and K in [16, 256], multiples of 16");
    const size_t smem = (size_t)(128 + N) * K * 2 + 16;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaFuncSetAttribute(k_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return check_launch("ocfd_tc_gemm_bf16 attribute");
    cudaMemsetAsync(ctx->d_error, 0, sizeof(uint32_t), st);
    k_tc_gemm<<<1, 128, smem, st>>>(A, B, C, N, K, ctx->d_error);
    ocfd_status s = check_launch("ocfd_tc_gemm_bf16");
    if (s != OCFD_OK) return s;
    uint32_t e = 0;
    if (cudaMemcpyAsync(&e, ctx->d_error, sizeof(e), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return check_launch("ocfd_tc_gemm_bf16");
    if (e) return fail(OCFD_TIMEOUT, "ocfd_tc_gemm_bf16: the MMA completion wait ran out");
    return OCFD_OK;
}
