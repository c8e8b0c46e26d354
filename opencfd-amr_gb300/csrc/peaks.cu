// FP64 / FP32 FMA throughput probe: register-only dependent FMA chains, several
// independent chains per thread, enough CTAs to fill every SM.  The result is
// the denominator of the FP64/FP32 pipe-utilisation figures (the HBM and bf16
// peaks come from elsewhere).
#include <cuda_runtime.h>

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

}  // namespace ocfd

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
