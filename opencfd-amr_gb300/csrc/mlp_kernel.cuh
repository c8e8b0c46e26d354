// The chemistry surrogate network's fused tile routine (5 layers on the tensor
// cores for 128 rows), shared by the training kernels (mlp.cu) and the solver's
// surrogate chemistry substep (chem.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "ocfd/ocfd.h"
#include "tcgen05.cuh"

namespace ocfd {

using namespace tc;

__device__ __forceinline__ uint16_t bf16_bits(float x) {  // round to nearest even
    const uint32_t u = __float_as_uint(x);
    if ((u & 0x7f800000u) == 0x7f800000u) return (uint16_t)((u >> 16) | ((u & 0xffffu) ? 0x40u : 0u));
    return (uint16_t)((u + 0x7fffu + ((u >> 16) & 1u)) >> 16);
}

__host__ __device__ __forceinline__ uint32_t tmem_cols(int n) {
    uint32_t c = 32;
    while ((int)c < n) c <<= 1;
    return c;
}

// ============================================================ the network
// 12 inputs (T, p, 9 Y, log10 dt), 4 hidden layers of 128 with GELU, 10 outputs
// (increments of T and of the 9 Y).  Layer l has W_l [N_l x K_l] (out x in,
// row-major BF16) and b_l [N_l] (FP32); the input is padded to K_1 = 16 and the
// output to N_5 = 16 with zero weights.
constexpr int MLP_IN = 12, MLP_OUT = 10, MLP_H = 128;
__host__ __device__ constexpr int LN(int l) { return l == 4 ? 16 : 128; }                  // outputs of layer l
__host__ __device__ constexpr int LK(int l) { return l == 0 ? 16 : 128; }                  // inputs of layer l
__host__ __device__ constexpr int WOFF(int l) { return l == 0 ? 0 : 2048 + (l - 1) * 16384; }  // element offset of W_l
constexpr int WTOT = 53248;
__host__ __device__ constexpr int BOFF(int l) { return 128 * l; }
constexpr int BTOT = 528;
// shared memory of the fused kernel (bytes)
constexpr int S_W = 0;                        // the five B operands, K-major, as WOFF * 2
constexpr int S_A0 = WTOT * 2;                // 128 x 16 input operand
constexpr int S_H = S_A0 + 128 * 16 * 2;      // 128 x 128 hidden operand
constexpr int S_B = S_H + 128 * 128 * 2;      // biases, FP32
constexpr int S_BAR = S_B + BTOT * 4;
constexpr int S_TOT = S_BAR + 16;

struct MlpNet {
    const uint16_t* W;  // BF16 weights, WTOT elements
    const float* b;     // FP32 biases, BTOT
    float in_mu[MLP_IN], in_isd[MLP_IN];     // feature normalisation: (x - mu) * isd
    float out_mu[MLP_OUT], out_sd[MLP_OUT];  // target scaling: y * sd + mu
    float out_scale[MLP_OUT];                // > 0: y is sign(r) log1p(|r| / scale) of the rate r
};

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }

// stage the weights (K-major B operands) and biases of the network
__device__ __forceinline__ void mlp_stage_weights(const MlpNet& net, unsigned char* sm) {
    for (int l = 0; l < 5; ++l) {
        const int N = LN(l), K = LK(l);
        unsigned char* dst = sm + S_W + WOFF(l) * 2;
        const uint16_t* src = net.W + WOFF(l);
        // 8 consecutive k of a row are one 16-byte core-matrix row in both layouts
        // (W and every WOFF(l) * 2 are 16-byte aligned)
        for (int q = threadIdx.x; q < N * K / 8; q += blockDim.x) {
            const int n = q / (K / 8), k = (q % (K / 8)) * 8;
            *reinterpret_cast<uint4*>(dst + kmajor_offset(n, k, N)) =
                __ldg(reinterpret_cast<const uint4*>(src + (long long)n * K + k));
        }
    }
    float* sb = reinterpret_cast<float*>(sm + S_B);
    for (int e = threadIdx.x; e < BTOT; e += blockDim.x) sb[e] = net.b[e];
}

// warpgroups (of 128 threads) that share one 128-row tile: the bias + GELU
// epilogue of a hidden layer (128 columns per row, erf and BF16 packing per
// element) takes far longer than the layer's MMAs, so it is split over MLP_G
// warpgroups by columns
constexpr int MLP_G = 4;

// one 128-row tile through the five layers; the input operand (S_A0) is staged.
// The CTA has 128 G threads: thread t serves row t % 128 (warp w reads TMEM
// lanes 32 (w % 4) .. 32 (w % 4) + 31) and columns [(t / 128) 128 / G,
// (t / 128 + 1) 128 / G) of every hidden layer; the output layer's 16 columns go
// to the first warpgroup (out[]).  Hidden activations go to `zs` / `hs` (FP32
// pre-activations, BF16 activations; may be null).  Returns false when an MMA
// completion wait ran out.
template <int G>
__device__ __forceinline__ bool mlp_tile(unsigned char* sm, uint32_t tbase, uint64_t* bar, uint32_t& phase,
                                         float* out, float* zs, uint16_t* hs, long long ld) {
    static_assert(G == 1 || G == 2 || G == 4, "warpgroups per tile");
    constexpr int CW = MLP_H / G;
    const int tid = threadIdx.x, row = tid & 127, cg = tid >> 7;
    const float* sb = reinterpret_cast<const float*>(sm + S_B);
    const uint32_t trow = tbase + ((uint32_t)(((tid >> 5) & 3) * 32) << 16);
    for (int l = 0; l < 5; ++l) {
        fence_async_smem();
        fence_before_sync();
        __syncthreads();
        fence_after_sync();
        if (tid == 0) {
            const uint32_t idesc = idesc_bf16_f32(128, LN(l));
            const unsigned char* A = sm + (l == 0 ? S_A0 : S_H);
            const unsigned char* B = sm + S_W + WOFF(l) * 2;
            for (int ks = 0; ks < LK(l) / 16; ++ks)
                mma_bf16(tbase, smem_desc(smem_u32(A + ks * 128 * 32)), smem_desc(smem_u32(B + ks * LN(l) * 32)),
                         idesc, ks > 0 ? 1u : 0u);
            mma_commit(bar);
        }
        const bool ok = mbar_wait(bar, phase);
        phase ^= 1u;
        fence_after_sync();
        if (!ok) return false;
        if (l < 4) {
            // bias + GELU, BF16 into the hidden operand: 8 consecutive columns of a
            // row are one 16-byte core-matrix row, stored at once
            for (int c0 = cg * CW; c0 < (cg + 1) * CW; c0 += 32) {
                float v[32];
                tmem_ld32(trow + (uint32_t)c0, v);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    uint32_t pk[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int i = q * 8 + e * 2;
                        const float z0 = v[i] + sb[BOFF(l) + c0 + i], z1 = v[i + 1] + sb[BOFF(l) + c0 + i + 1];
                        pk[e] = (uint32_t)bf16_bits(gelu(z0)) | ((uint32_t)bf16_bits(gelu(z1)) << 16);
                        if (zs) {
                            float* zr = zs + (long long)l * 128 * ld + (long long)row * 128 + c0 + i;
                            zr[0] = z0;
                            zr[1] = z1;
                        }
                    }
                    const uint4 w = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                    *reinterpret_cast<uint4*>(sm + S_H + kmajor_offset(row, c0 + q * 8, 128)) = w;
                    if (hs)
                        *reinterpret_cast<uint4*>(hs + (long long)l * 128 * ld + (long long)row * 128 + c0 + q * 8) = w;
                }
            }
        } else if (cg == 0) {
            float v[16];
            tmem_ld16(trow, v);
#pragma unroll
            for (int i = 0; i < 16; ++i) out[i] = v[i] + sb[BOFF(4) + i];
        }
    }
    return true;
}

// the device view of a network object (mlp.cu)
MlpNet mlp_net(const ocfd_mlp* n);

}  // namespace ocfd
