// FP64 / FP32 FMA throughput probe: register-only dependent FMA chains, several
// independent chains per thread, enough CTAs to fill every SM.  The result is
// the denominator of the FP64/FP32 pipe-utilisation figures (the HBM and bf16
// peaks come from elsewhere).  Also the packed FP32 rate (FFMA2, two lanes per
// instruction, which the mixed form's WENO-Z issues) and a check of the FP64
// reciprocal the fused FP64 kernels use in place of IEEE division.
#include <cuda_runtime.h>

#include "device_physics.cuh"
#include "ocfd_internal.h"

namespace ocfd {

template <class T, int CHAINS>
__global__ void k_fma_chain(T* out, int iters, T a, T b) {
    T x[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) x[c] = (T)(threadIdx.x + c);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < CHAINS; ++c) x[c] = x[c] * a + b;
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s += x[c];
    if (s == (T)-12345.678) out[blockIdx.x] = s;  // keeps the chains alive
}

template <int CHAINS>
__global__ void k_ffma2_chain(float2* out, int iters, float2 a, float2 b) {
    float2 x[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) x[c] = make_float2((float)(threadIdx.x + c), (float)(threadIdx.x - c));
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < CHAINS; ++c) x[c] = __ffma2_rn(x[c], a, b);
    }
    float s = 0;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s += x[c].x + x[c].y;
    if (s == -12345.678f) out[blockIdx.x] = x[0];
}

__global__ void k_rcp_check(const double* __restrict__ x, double* __restrict__ fast, double* __restrict__ ieee,
                            long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        fast[i] = rcp_nr(x[i]);
        ieee[i] = 1.0 / x[i];
    }
}

template <class T, int CHAINS>
static double time_fma(int sms) {
    T* out = nullptr;
    if (cudaMalloc(&out, sizeof(T) * sms * 8) != cudaSuccess) return -1;
    const int threads = 256, blocks = sms * 8, iters = 4096;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fma_chain<T, CHAINS><<<blocks, threads>>>(out, 64, (T)0.999, (T)0.001);  // warm-up
    cudaEventRecord(e0);
    k_fma_chain<T, CHAINS><<<blocks, threads>>>(out, iters, (T)0.999, (T)0.001);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    double flops = 2.0 * CHAINS * (double)iters * threads * blocks;
    return flops / (ms * 1e-3) / 1e9;
}

template <int CHAINS>
static double time_ffma2(int sms) {
    float2* out = nullptr;
    if (cudaMalloc(&out, sizeof(float2) * sms * 8) != cudaSuccess) return -1;
    const int threads = 256, blocks = sms * 8, iters = 4096;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const float2 a = make_float2(0.999f, 0.998f), b = make_float2(0.001f, 0.002f);
    k_ffma2_chain<CHAINS><<<blocks, threads>>>(out, 64, a, b);
    cudaEventRecord(e0);
    k_ffma2_chain<CHAINS><<<blocks, threads>>>(out, iters, a, b);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    double flops = 4.0 * CHAINS * (double)iters * threads * blocks;   // 2 lanes x 2 flops per FFMA2
    return flops / (ms * 1e-3) / 1e9;
}

}  // namespace ocfd

extern "C" ocfd_status ocfd_measure_ffma2_peak(double* fp32x2_gflops) {
    int dev = 0, sms = 0;
    if (!fp32x2_gflops) return ocfd::fail(OCFD_BAD_ARG, "ocfd_measure_ffma2_peak: null argument");
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return ocfd::fail(OCFD_NO_DEVICE, "ocfd_measure_ffma2_peak: no device");
    }
    *fp32x2_gflops = ocfd::time_ffma2<8>(sms);
    return ocfd::check_launch("ocfd_measure_ffma2_peak");
}

extern "C" ocfd_status ocfd_check_rcp_f64(const double* x, double* fast, double* ieee, int64_t n, void* stream) {
    if (!x || !fast || !ieee || n < 0) return ocfd::fail(OCFD_BAD_ARG, "ocfd_check_rcp_f64: bad argument");
    if (n == 0) return OCFD_OK;
    const long long blocks = (n + 255) / 256;
    ocfd::k_rcp_check<<<(int)(blocks < 4096 ? blocks : 4096), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        x, fast, ieee, n);
    return ocfd::check_launch("ocfd_check_rcp_f64");
}

extern "C" ocfd_status ocfd_measure_fma_peaks(double* fp64_gflops, double* fp32_gflops) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return ocfd::fail(OCFD_NO_DEVICE, "ocfd_measure_fma_peaks: no device");
    }
    if (fp64_gflops) *fp64_gflops = ocfd::time_fma<double, 8>(sms);
    if (fp32_gflops) *fp32_gflops = ocfd::time_fma<float, 8>(sms);
    return ocfd::check_launch("ocfd_measure_fma_peaks");
}
