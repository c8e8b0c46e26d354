// FP32 building blocks of the mixed-precision forms: WENO-Z on a normalised
// stencil and FP64 <-> FP32 conversions on the integer pipes.  Used by the
// regular-box kernel (rhs_regular_kernel.cuh) and the multispecies faces (chem.cu).
#pragma once

#include <cuda_runtime.h>

namespace ocfd {

// WENO-Z in FP32.  The stencil values are normalised by the power of two s
// nearest above their largest magnitude (an exact scaling), and the reference's
// absolute smoothness epsilon (1e-6, Reconstruction.H:83) is rescaled to the
// local state as eps / s^2 in the normalised units.  The scheme is therefore
// the FP64 scheme up to FP32 rounding, and no smoothness indicator can overflow
// whatever the magnitude of the flux.
__device__ __forceinline__ float wenoz_side_f(float V1, float V2, float V3, float V4, float V5, float eps) {
    float s11 = (13.0f / 12.0f) * (V1 - 2.0f * V2 + V3) * (V1 - 2.0f * V2 + V3) +
                0.25f * (V1 - 4.0f * V2 + 3.0f * V3) * (V1 - 4.0f * V2 + 3.0f * V3);
    float s22 = (13.0f / 12.0f) * (V2 - 2.0f * V3 + V4) * (V2 - 2.0f * V3 + V4) + 0.25f * (V2 - V4) * (V2 - V4);
    float s33 = (13.0f / 12.0f) * (V3 - 2.0f * V4 + V5) * (V3 - 2.0f * V4 + V5) +
                0.25f * (3.0f * V3 - 4.0f * V4 + V5) * (3.0f * V3 - 4.0f * V4 + V5);
    const float s55 = fabsf(s11 - s33);
    // tau / (eps + beta), capped at 1e18: a stencil side that is exactly flat
    // (beta = 0) next to a jump gives tau / eps, which for |V| above ~1e5 in
    // normalised units of a small eps would overflow (1 + r^2) in FP32; at the cap
    // that side's weight already dominates the others by > 1e30
    const float r1 = fminf(__fdividef(s55, eps + s11), 1e18f), r2 = fminf(__fdividef(s55, eps + s22), 1e18f),
                r3 = fminf(__fdividef(s55, eps + s33), 1e18f);
    const float a1 = 1.0f + r1 * r1, a2 = 6.0f * (1.0f + r2 * r2), a3 = 3.0f * (1.0f + r3 * r3);
    const float v1 = 2.0f * V1 - 7.0f * V2 + 11.0f * V3;
    const float v2 = -V2 + 5.0f * V3 + 2.0f * V4;
    const float v3 = 2.0f * V3 + 5.0f * V4 - V5;
    return __fdividef(a1 * v1 + a2 * v2 + a3 * v3, 6.0f * (a1 + a2 + a3));
}

// f+ at cells i-3..i+1, or f- at i+2..i-2 (the mirrored stencil): normalise,
// reconstruct, scale back
__device__ __forceinline__ float wenoz_norm_f(float V1, float V2, float V3, float V4, float V5) {
    const float m = fmaxf(fmaxf(fmaxf(fabsf(V1), fabsf(V2)), fmaxf(fabsf(V3), fabsf(V4))), fabsf(V5));
    const int ex = (__float_as_int(m) >> 23) & 0xff;
    // zero / subnormal stencils, and inf / NaN, are reconstructed as they are
    if (ex == 0 || ex > 250) return wenoz_side_f(V1, V2, V3, V4, V5, 1e-6f);
    const float sc = __int_as_float((254 - ex) << 23);      // 2^-(ex-127)
    const float inv = __int_as_float(ex << 23);             // 2^(ex-127)
    // 1e-6 absolute, in normalised units; kept > 0 so that 0/0 cannot occur
    const float eps = fmaxf(1e-6f * sc * sc, 1e-37f);
    return wenoz_side_f(V1 * sc, V2 * sc, V3 * sc, V4 * sc, V5 * sc, eps) * inv;
}

// Conversions between FP64 and FP32 on the integer pipes.  GB300 runs FP64
// (and its conversions) at 2 instructions / cycle / SM, so in the mixed form the
// state is narrowed and the FP32 divergence widened with bit operations:
// double -> float truncates the mantissa (error < 1 ulp of float; values below
// 2^-126 flush to zero), float -> double is exact.
__device__ __forceinline__ float d2f_bits(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const unsigned sign = hi & 0x80000000u;
    const int ed = (int)((hi >> 20) & 0x7ffu);
    const int e = ed - 896;  // rebias 1023 -> 127
    const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    unsigned f;
    if (e <= 0) f = sign;
    else if (ed == 0x7ff) f = sign | 0x7f800000u | ((((hi & 0xfffffu) | lo) != 0u) ? 0x400000u : 0u);
    else if (e >= 255) f = sign | 0x7f800000u;
    else f = sign | ((unsigned)e << 23) | m;
    return __uint_as_float(f);
}

__device__ __forceinline__ double f2d_bits(float x) {
    const unsigned u = __float_as_uint(x);
    const unsigned sign = u & 0x80000000u, e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    unsigned hi, lo = 0u;
    if (e == 0u) hi = sign;
    else if (e == 0xffu) hi = sign | 0x7ff00000u | (m ? 0x80000u : 0u);
    else {
        hi = sign | ((e + 896u) << 20) | (m >> 3);
        lo = m << 29;
    }
    return __hiloint2double((int)hi, (int)lo);
}

}  // namespace ocfd
