// Cut-cell (embedded boundary) point physics on the GPU, in the operation order
// of Source/EB/EBkernels.H and Source/EB/EBdiffusion.H.
#pragma once

#include "device_physics.cuh"

namespace ocfd {

// EBCellFlag: bits 0-1 type, neighbour (i,j,k) at bit 4 + (i+1) + 3(j+1) + 9(k+1).
// The reference queries offsets of -2 (EBkernels.H:22,43,64); those map to the
// same linear bit position, and to "not connected" outside the word.
__device__ __forceinline__ bool eb_conn(uint32_t f, int i, int j, int k) {
    const int p = 4 + (i + 1) + 3 * (j + 1) + 9 * (k + 1);
    return p >= 0 && p < 32 && ((f >> p) & 1u);
}
__device__ __forceinline__ bool eb_covered(uint32_t f) { return (f & 3u) == 3u; }
__device__ __forceinline__ bool eb_regular(uint32_t f) { return (f & 3u) == 0u; }

// minmod, Source/kernel/Reconstruction.H:8-19 (T = double: the reference's
// arithmetic; T = float: the mixed form's cut-cell faces)
template <class T>
__device__ __forceinline__ T minmod(T a, T b) {
    if (a * b > 0) return fabs(a) > fabs(b) ? b : a;
    return T(0);
}
// FP64: the same selections with both tests on the integer pipes (GB300's FP64
// pipe, two instructions per cycle per SM, also executes FP64 multiplies and
// comparisons).  a b > 0 is: both non-zero with equal sign bits; |x|'s bits order
// as |x| does.  The selections differ from the reference's only for NaN operands,
// which the flow never carries, and where a b underflows to 0 (|a b| below
// 5e-324), where the slope selected is below the last bit of any state value.
template <>
__device__ __forceinline__ double minmod<double>(double a, double b) {
    const long long mag = 0x7fffffffffffffffLL;
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    const long long ma = ia & mag, mb = ib & mag;
    if ((ia ^ ib) >= 0 && ma != 0 && mb != 0) return ma > mb ? b : a;
    return 0.0;
}

// eb_recon_x/y/z for one component: left/right states at the D-face of cell c
// given the values at c-2e, c-e, c, c+e and the flag of c.
template <class T>
__device__ __forceinline__ void eb_recon(uint32_t f, int D, T vm2, T vm1, T v0, T vp1, T& l, T& r) {
    const int di = D == 0, dj = D == 1, dk = D == 2;
    l = vm1;
    r = v0;
    if (eb_conn(f, -di, -dj, -dk)) {
        if (eb_conn(f, -2 * di, -2 * dj, -2 * dk)) l = vm1 + T(0.5) * minmod<T>(v0 - vm1, vm1 - vm2);
        if (eb_conn(f, di, dj, dk)) r = v0 - T(0.5) * minmod<T>(vp1 - v0, v0 - vm1);
    }
}

// 1/x: the Newton-refined reciprocal in FP64 (device_physics.cuh), a plain
// division in FP32
template <class T>
__device__ __forceinline__ T recip(T x);
template <>
__device__ __forceinline__ double recip<double>(double x) { return rcp_nr(x); }
template <>
__device__ __forceinline__ float recip<float>(float x) { return 1.0f / x; }

// Van Leer flux vector splitting, Source/EB/EBkernels.H:73-171.  The reference's
// divisions become two reciprocals per face (the Mach numbers) and three
// constants of gamma: rg = 1/gamma (the /gamma of the normal momentum),
// rg21 = 1/(2(gamma^2 - 1)) and ggm1 = gamma/(gamma - 1); the same values to
// within a few ulps (FP64 parity of the cut-cell paths: 1e-12 per right-hand
// side).  The ideal-gas paths pass the constants formed once on the host
// (DevParm::vl_*); vanleer() forms them per face for a face-varying gamma.
template <class T>
__device__ __forceinline__ void vanleer_g(T smallp, T gamma, T rg, T rg21, T ggm1, const T* ql, const T* qr, int D,
                                          T* flx) {
    T fp[5] = {0, 0, 0, 0, 0}, fm[5] = {0, 0, 0, 0, 0};
    const T dl = ql[QRHO], ul = ql[QU], vl = ql[QV], wl = ql[QW], pl = ql[QPRES] > smallp ? ql[QPRES] : smallp;
    const T dr = qr[QRHO], ur = qr[QU], vr = qr[QV], wr = qr[QW], pr = qr[QPRES] > smallp ? qr[QPRES] : smallp;
    const T cL = ql[QC], cR = qr[QC];
    const int nn[3] = {D == 0, D == 1, D == 2};
    const T UL = D == 0 ? ul : (D == 1 ? vl : wl);
    const T UR = D == 0 ? ur : (D == 1 ? vr : wr);
    const T ML = UL * recip<T>(cL), MR = UR * recip<T>(cR);
    const T lv[3] = {ul, vl, wl}, rv[3] = {ur, vr, wr};
    if (ML >= T(1)) {
        fp[0] = dl * UL;
#pragma unroll
        for (int m = 0; m < 3; ++m) fp[1 + m] = dl * UL * lv[m] + T(nn[m]) * pl;
        fp[4] = UL * (ggm1 * pl + T(0.5) * dl * (ul * ul + vl * vl + wl * wl));
    } else if (fabs(ML) < T(1)) {
        const T Mp = T(0.25) * (T(1) + ML) * (T(1) + ML);
        const T t0 = dl * cL * Mp;
        fp[0] = t0;
#pragma unroll
        for (int m = 0; m < 3; ++m) fp[1 + m] = t0 * (nn[m] ? (-UL + T(2) * cL) * rg + lv[m] : lv[m]);
        fp[4] = t0 * (((gamma - 1) * UL + 2 * cL) * ((gamma - 1) * UL + 2 * cL) * rg21 +
                      (ul * ul + vl * vl + wl * wl - UL * UL) * T(0.5));
    }
    if (fabs(MR) < T(1)) {
        const T Mm = T(-0.25) * (MR - T(1)) * (MR - T(1));
        const T t0 = dr * cR * Mm;
        fm[0] = t0;
#pragma unroll
        for (int m = 0; m < 3; ++m) fm[1 + m] = t0 * (nn[m] ? (-UR - T(2) * cR) * rg + rv[m] : rv[m]);
        fm[4] = t0 * (((gamma - 1) * UR - 2 * cR) * ((gamma - 1) * UR - 2 * cR) * rg21 +
                      (ur * ur + vr * vr + wr * wr - UR * UR) * T(0.5));
    } else if (MR <= T(-1)) {
        fm[0] = dr * UR;
#pragma unroll
        for (int m = 0; m < 3; ++m) fm[1 + m] = dr * UR * rv[m] + T(nn[m]) * pr;
        fm[4] = UR * (ggm1 * pr + T(0.5) * dr * (ur * ur + vr * vr + wr * wr));
    }
#pragma unroll
    for (int n = 0; n < 5; ++n) flx[n] = fp[n] + fm[n];
}
template <class T>
__device__ __forceinline__ void vanleer(T smallp, T gamma, const T* ql, const T* qr, int D, T* flx) {
    vanleer_g<T>(smallp, gamma, recip<T>(gamma), recip<T>(2 * (gamma * gamma - 1)), gamma * recip<T>(gamma - T(1)),
                 ql, qr, D, flx);
}

// connectivity-aware transverse derivative of component `m` of q along t at the
// D-face of cell (i,j,k), Source/EB/EBdiffusion.H:36-58
__device__ __forceinline__ double eb_tderiv(const View<const double>& q, const View<const uint32_t>& flag,
                                            int m, int D, int t, int i, int j, int k, double dxinv_t) {
    const double weights[3] = {0., 1., 0.5};
    const int ti = t == 0, tj = t == 1, tk = t == 2;
    const int li = i - (D == 0), lj = j - (D == 1), lk = k - (D == 2);
    const uint32_t fh = flag(i, j, k), fl = flag(li, lj, lk);
    const int hip = eb_conn(fh, ti, tj, tk), him = eb_conn(fh, -ti, -tj, -tk);
    const int lop = eb_conn(fl, ti, tj, tk), lom = eb_conn(fl, -ti, -tj, -tk);
    const double whi = weights[hip + him], wlo = weights[lop + lom];
    return (0.5 * dxinv_t) *
           ((q(i + hip * ti, j + hip * tj, k + hip * tk, m) - q(i - him * ti, j - him * tj, k - him * tk, m)) * whi +
            (q(li + lop * ti, lj + lop * tj, lk + lop * tk, m) - q(li - lom * ti, lj - lom * tj, lk - lom * tk, m)) * wlo);
}

// eb_compute_visc_x/y/z (Source/EB/EBdiffusion.H:8-203); with `multi` the
// multispecies form of Source/CHEM/ChemViscous.H:357-575 (face mu / lambda
// given, species-enthalpy flux subtracted).  f points at component 0 of the
// face flux, fs is the component stride.
__device__ __forceinline__ void eb_visc_face(const DevParm& P, const View<const double>& q,
                                             const View<const uint32_t>& flag, int D, int i, int j,
                                             int k, const double* dxinv, double* f, long long fs,
                                             bool multi, double mu_f, double lam_f, double hflux) {
    const int li = i - (D == 0), lj = j - (D == 1), lk = k - (D == 2);
    const double Tc = q(i, j, k, QT), Tm = q(li, lj, lk, QT);
    double muf, ksum = 0;
    if (!multi) {
        const double mutl = sutherland(P, Tc), mutr = sutherland(P, Tm);
        muf = 0.5 * (mutl + mutr);
        ksum = mutl * P.kOverMu + mutr * P.kOverMu;
    } else {
        muf = mu_f;
    }
    const double dT = (Tc - Tm) * dxinv[D];
    double g[3][3];
#pragma unroll
    for (int m = 0; m < 3; ++m) g[m][D] = (q(i, j, k, QU + m) - q(li, lj, lk, QU + m)) * dxinv[D];
#pragma unroll
    for (int t = 0; t < 3; ++t) {
        if (t == D) continue;
        g[D][t] = eb_tderiv(q, flag, QU + D, D, t, i, j, k, dxinv[t]);
        g[t][t] = eb_tderiv(q, flag, QU + t, D, t, i, j, k, dxinv[t]);
    }
    const double divu = g[0][0] + g[1][1] + g[2][2];
    double tau[3];
#pragma unroll
    for (int m = 0; m < 3; ++m)
        tau[m] = (m == D) ? muf * (2.0 * g[D][D] - P.twoThirds * divu) : muf * (g[m][D] + g[D][m]);
#pragma unroll
    for (int m = 0; m < 3; ++m) f[(1 + m) * fs] += -tau[m];
    const double ub0 = q(i, j, k, QU) + q(li, lj, lk, QU);
    const double ub1 = q(i, j, k, QV) + q(li, lj, lk, QV);
    const double ub2 = q(i, j, k, QW) + q(li, lj, lk, QW);
    if (!multi)
        f[4 * fs] += -0.5 * (ub0 * tau[0] + ub1 * tau[1] + ub2 * tau[2] + ksum * dT);
    else
        f[4 * fs] += -0.5 * (ub0 * tau[0] + ub1 * tau[1] + ub2 * tau[2]) - lam_f * dT - hflux;
}

}  // namespace ocfd
