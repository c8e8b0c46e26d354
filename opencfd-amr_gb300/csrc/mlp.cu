// Chemistry surrogate network on the 5th-generation tensor cores: BF16 weights
// and activations, FP32 accumulation in tensor memory (tcgen05.mma, TMEM),
// operands staged in shared memory (tcgen05.cuh for the layouts).
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "ocfd_internal.h"
#include "tcgen05.cuh"

namespace ocfd {

using namespace tc;

static __device__ __forceinline__ uint16_t bf16_bits(float x) {  // round to nearest even
    const uint32_t u = __float_as_uint(x);
    if ((u & 0x7f800000u) == 0x7f800000u) return (uint16_t)((u >> 16) | ((u & 0xffffu) ? 0x40u : 0u));
    return (uint16_t)((u + 0x7fffu + ((u >> 16) & 1u)) >> 16);
}

static __host__ __device__ __forceinline__ uint32_t tmem_cols(int n) {
    uint32_t c = 32;
    while ((int)c < n) c <<= 1;
    return c;
}

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

}  // namespace ocfd

using namespace ocfd;

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
