// FP32 building blocks of the mixed-precision forms: WENO-Z on a normalised
// stencil and FP64 <-> FP32 conversions on the integer pipes.  Used by the
// regular-box kernel (rhs_regular_kernel.cuh) and the multispecies faces (chem.cu).
#pragma once

#include <cuda_runtime.h>

namespace ocfd {

// WENO-Z in FP32.  The stencil values of a face (its f+ and f- stencils) are
// normalised by the power of two s nearest above their largest magnitude (an
// exact scaling), and the reference's
// absolute smoothness epsilon (1e-6, Reconstruction.H:83) is rescaled to the
// local state as eps / s^2 in the normalised units.  The scheme is therefore
// the FP64 scheme up to FP32 rounding, and no smoothness indicator can overflow
// whatever the magnitude of the flux.
//
// A face flux is the f+ reconstruction plus the f- one, two independent
// evaluations of the same expressions: they run as the two lanes of float2
// values, so that every add / multiply / FMA of the scheme is one packed FP32
// instruction (sm_100 and later) for both sides.  Only the approximate
// reciprocals and the ratio cap are per lane.

__device__ __forceinline__ float2 p_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 p_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 p_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 p_set(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 p_rcp(float2 a) { return make_float2(__fdividef(1.0f, a.x), __fdividef(1.0f, a.y)); }

// Normalisation of a face's two stencils by one power of two: the scale sc,
// its inverse and 4 epsilon in normalised units (the smoothness indicators are
// carried as 4 beta, see wenoz_pm_f).  Zero / subnormal stencils, and inf /
// NaN, are reconstructed as they are (sc = 1, epsilon 1e-6).
__device__ __forceinline__ void wenoz_scale(float m, float& sc, float& inv, float& eps4) {
    const int ex = (__float_as_int(m) >> 23) & 0xff;
    const bool plain = ex == 0 || ex > 250;
    sc = plain ? 1.0f : __int_as_float((254 - ex) << 23);   // 2^-(ex-127)
    inv = plain ? 1.0f : __int_as_float(ex << 23);          // 2^(ex-127)
    // 4 x 1e-6 absolute, in normalised units; kept > 0 so that 0/0 cannot occur
    eps4 = plain ? 4e-6f : fmaxf(4e-6f * sc * sc, 4e-37f);
}

// f+ at cells i-3..i+1 (a1..a5) plus f- at i+2..i-2 (b1..b5, the mirrored
// stencil): the WENO-Z face flux.  The smoothness indicators are carried as
// 4 beta_k = (13/3) d_k^2 + e_k^2 with the epsilon scaled by 4 (an exact
// scaling that leaves tau / (eps + beta_k) unchanged), and with the weights
// alpha_k = d_k W_k, W_k = 1 + (tau / (eps + beta_k))^2, d = (1, 6, 3), the face
// value sum alpha_k v_k / (6 sum alpha_k) is formed as
// (W_1 v_1 / 6 + W_2 v_2 + W_3 v_3 / 2) / (W_1 + 6 W_2 + 3 W_3), the 1/6 and
// the d_k folded into the candidate polynomials' coefficients.
__device__ __forceinline__ float wenoz_pm_f(float a1, float a2, float a3, float a4, float a5, float b1,
                                            float b2, float b3, float b4, float b5) {
    const float ma = fmaxf(fmaxf(fmaxf(fabsf(a1), fabsf(a2)), fmaxf(fabsf(a3), fabsf(a4))), fabsf(a5));
    const float mb = fmaxf(fmaxf(fmaxf(fabsf(b1), fabsf(b2)), fmaxf(fabsf(b3), fabsf(b4))), fabsf(b5));
    float s, iv, e4;
    wenoz_scale(fmaxf(ma, mb), s, iv, e4);
    const float2 sc = p_set(s), eps4 = p_set(e4);
    const float2 V1 = p_mul(make_float2(a1, b1), sc), V2 = p_mul(make_float2(a2, b2), sc),
                 V3 = p_mul(make_float2(a3, b3), sc), V4 = p_mul(make_float2(a4, b4), sc),
                 V5 = p_mul(make_float2(a5, b5), sc);
    const float2 c133 = p_set(13.0f / 3.0f), m1 = p_set(-1.0f), m2 = p_set(-2.0f), m4 = p_set(-4.0f),
                 c2 = p_set(2.0f), c3 = p_set(3.0f), c5 = p_set(5.0f);
    // Jiang-Shu smoothness indicators (Reconstruction.H:70-139), times 4
    const float2 d1 = p_fma(m2, V2, p_add(V1, V3));           // V1 - 2 V2 + V3
    const float2 e1 = p_fma(c3, V3, p_fma(m4, V2, V1));       // V1 - 4 V2 + 3 V3
    const float2 s1 = p_fma(p_mul(c133, d1), d1, p_mul(e1, e1));
    const float2 d2 = p_fma(m2, V3, p_add(V2, V4));           // V2 - 2 V3 + V4
    const float2 e2 = p_fma(m1, V4, V2);                      // V2 - V4
    const float2 s2 = p_fma(p_mul(c133, d2), d2, p_mul(e2, e2));
    const float2 d3 = p_fma(m2, V4, p_add(V3, V5));           // V3 - 2 V4 + V5
    const float2 e3 = p_fma(c3, V3, p_fma(m4, V4, V5));       // 3 V3 - 4 V4 + V5
    const float2 s3 = p_fma(p_mul(c133, d3), d3, p_mul(e3, e3));
    // tau / (eps + beta) with tau = |beta_1 - beta_3|, capped at 1e18: a stencil
    // side that is exactly flat (beta = 0) next to a jump gives tau / eps, which
    // for |V| above ~1e5 in normalised units of a small eps would overflow
    // (1 + r^2) in FP32; at the cap that side's weight already dominates the
    // others by > 1e30
    const float2 tau = p_fma(m1, s3, s1);
    float2 r1 = p_mul(tau, p_rcp(p_add(eps4, s1))), r2 = p_mul(tau, p_rcp(p_add(eps4, s2))),
           r3 = p_mul(tau, p_rcp(p_add(eps4, s3)));
    r1 = make_float2(fminf(fabsf(r1.x), 1e18f), fminf(fabsf(r1.y), 1e18f));
    r2 = make_float2(fminf(fabsf(r2.x), 1e18f), fminf(fabsf(r2.y), 1e18f));
    r3 = make_float2(fminf(fabsf(r3.x), 1e18f), fminf(fabsf(r3.y), 1e18f));
    const float2 one = p_set(1.0f);
    const float2 w1 = p_fma(r1, r1, one), w2 = p_fma(r2, r2, one), w3 = p_fma(r3, r3, one);
    // candidate stencils v_1 / 6, v_2, v_3 / 2
    const float2 v1 = p_fma(p_set(11.0f / 6.0f), V3, p_fma(p_set(-7.0f / 6.0f), V2, p_mul(p_set(1.0f / 3.0f), V1)));
    const float2 v2 = p_fma(c2, V4, p_fma(c5, V3, p_mul(m1, V2)));
    const float2 v3 = p_fma(p_set(-0.5f), V5, p_fma(p_set(2.5f), V4, V3));
    const float2 num = p_fma(w1, v1, p_fma(w2, v2, p_mul(w3, v3)));
    const float2 den = p_fma(c3, w3, p_fma(p_set(6.0f), w2, w1));
    const float2 f = p_mul(num, p_rcp(den));
    return (f.x + f.y) * iv;
}

// Steger-Warming split in FP32 (FluxSplit.H:11-193) in the grouping of the FP64
// sw_split_d: qt = ua^2 + ub^2 of the tangential velocities shared by the
// |.|^2 terms, the energy flux as E1 v2 + E2 (vvc1 + w2) + E3 (vvc2 + w2), the
// tangential momentum fluxes as the mass flux times the velocity, and the
// eigenvalue parts (x + |x|)/2, x - (x + |x|)/2 as the exact max(x, 0),
// min(x, 0).  Every rounding is written out: __fmul_rn / __fadd_rn / __fsub_rn
// are never fused and __fmaf_rn always is, so the compiler has no choice left
// and the fluxes of a cell do not depend on the code around the call (primitives
// formed inline or reloaded from shared memory split to the same values).
template <int D>
__device__ __forceinline__ void sw_split_f32(float d, float u, float v, float w, float c, float t1, float t2,
                                             float t3, float gm1, float* fp, float* fm) {
    const float vel[3] = {u, v, w};
    const float un = vel[D], ua = vel[(D + 1) % 3], ub = vel[(D + 2) % 3];
    const float qt = __fmaf_rn(ub, ub, __fmul_rn(ua, ua));
    const float uc1 = __fsub_rn(un, c), uc2 = __fadd_rn(un, c);
    const float w2 = __fmul_rn(__fmul_rn(t3, c), c);
    const float v2 = __fmul_rn(gm1, __fmaf_rn(un, un, qt));
    const float h1 = __fmaf_rn(0.5f, __fmaf_rn(uc1, uc1, qt), w2);
    const float h2 = __fmaf_rn(0.5f, __fmaf_rn(uc2, uc2, qt), w2);
    const float E1P = fmaxf(un, 0.0f), E2P = fmaxf(uc1, 0.0f), E3P = fmaxf(uc2, 0.0f);
    const float E1M = fminf(un, 0.0f), E2M = fminf(uc1, 0.0f), E3M = fminf(uc2, 0.0f);
    const float t0 = __fmul_rn(d, t1);
    const float a1p = __fmul_rn(t2, E1P), a1m = __fmul_rn(t2, E1M);
    const float rp = __fmul_rn(t0, __fadd_rn(__fadd_rn(a1p, E2P), E3P));
    const float rm = __fmul_rn(t0, __fadd_rn(__fadd_rn(a1m, E2M), E3M));
    fp[0] = rp;
    fm[0] = rm;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        if (m == D) {
            fp[1 + m] = __fmul_rn(t0, __fmaf_rn(E3P, uc2, __fmaf_rn(E2P, uc1, __fmul_rn(a1p, un))));
            fm[1 + m] = __fmul_rn(t0, __fmaf_rn(E3M, uc2, __fmaf_rn(E2M, uc1, __fmul_rn(a1m, un))));
        } else {
            fp[1 + m] = __fmul_rn(rp, vel[m]);
            fm[1 + m] = __fmul_rn(rm, vel[m]);
        }
    }
    fp[4] = __fmul_rn(t0, __fmaf_rn(E3P, h2, __fmaf_rn(E2P, h1, __fmul_rn(E1P, v2))));
    fm[4] = __fmul_rn(t0, __fmaf_rn(E3M, h2, __fmaf_rn(E2M, h1, __fmul_rn(E1M, v2))));
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
