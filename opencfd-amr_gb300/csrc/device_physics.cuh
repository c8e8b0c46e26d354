// Point-level physics of the ideal-gas path, written for the GPU (and callable
// on the host: include/ocfd/compat.H builds the reference's per-point functions
// from them).  Each function keeps the operation order of the reference
// expression it replaces,
// so the FP64 kernels agree with the reference to rounding (the parity tests
// use 1e-12 norm-wise; differences come only from FMA contraction).
#pragma once

#include "ocfd_internal.h"

namespace ocfd {

enum { URHO = 0, UMX = 1, UMY = 2, UMZ = 3, UEDEN = 4, NCONS = 5 };
enum { QRHO = 0, QU = 1, QV = 2, QW = 3, QPRES = 4, QT = 5, QC = 6, QGAMA = 7 };

__host__ __device__ __forceinline__ double dmax(double a, double b) { return a > b ? a : b; }
__host__ __device__ __forceinline__ double dmin(double a, double b) { return a < b ? a : b; }

// c2prim, Source/kernel/Kernels.H:13-40.  q = rho, u, v, w, p, T, c.
__host__ __device__ __forceinline__ void c2prim_ideal(const DevParm& P, double u0, double u1, double u2,
                                             double u3, double u4, double* q) {
    double rho = dmax(u0, P.smallr);
    double rhoinv = 1.0 / rho;
    double ux = u1 * rhoinv, uy = u2 * rhoinv, uz = u3 * rhoinv;
    double kineng = 0.5 * (ux * ux + uy * uy + uz * uz);
    double ei = u4 - rho * kineng;
    double p = dmax((P.gamma - 1.0) * ei, P.smallp);
    double T = p / (rho * P.Rg);
    q[QRHO] = rho;
    q[QU] = ux;
    q[QV] = uy;
    q[QW] = uz;
    q[QPRES] = p;
    q[QT] = T;
    q[QC] = sqrt(P.gamma * P.Rg * T);
}

// Steger-Warming split along D (Source/kernel/FluxSplit.H:11-193), given the
// split constants t1 = 1/(2g), t2 = 2(g-1), t3 = (3-g)/(2(g-1)), gm1 = g-1.
// T = double keeps the reference's expressions; T = float serves the
// mixed-precision form.
template <int D, class T = double>
__host__ __device__ __forceinline__ void sw_split(T d, T u, T v, T w, T c, T t1, T t2, T t3, T gm1, T* fp,
                                         T* fm) {
    const T vel[3] = {u, v, w};
    const T un = vel[D];
    const T uc1 = un - c, uc2 = un + c;
    T a0 = u, a1 = v, a2 = w, b0 = u, b1 = v, b2 = w;
    if (D == 0) { a0 = uc1; b0 = uc2; }
    if (D == 1) { a1 = uc1; b1 = uc2; }
    if (D == 2) { a2 = uc1; b2 = uc2; }
    const T half = T(0.5);
    const T vvc1 = half * (a0 * a0 + a1 * a1 + a2 * a2);
    const T vvc2 = half * (b0 * b0 + b1 * b1 + b2 * b2);
    const T v2 = gm1 * (u * u + v * v + w * w);
    const T w2 = t3 * c * c;
    const T E1 = un, E2 = un - c, E3 = un + c;
    const T E1P = (E1 + fabs(E1)) * half, E2P = (E2 + fabs(E2)) * half, E3P = (E3 + fabs(E3)) * half;
    const T E1M = E1 - E1P, E2M = E2 - E2P, E3M = E3 - E3P;
    const T t0 = d * t1;
    const T sp = t2 * E1P + E2P + E3P, sm = t2 * E1M + E2M + E3M;
    fp[URHO] = t0 * sp;
    fm[URHO] = t0 * sm;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        if (m == D) {
            fp[UMX + m] = t0 * (t2 * E1P * un + E2P * uc1 + E3P * uc2);
            fm[UMX + m] = t0 * (t2 * E1M * un + E2M * uc1 + E3M * uc2);
        } else {
            fp[UMX + m] = t0 * vel[m] * sp;
            fm[UMX + m] = t0 * vel[m] * sm;
        }
    }
    fp[UEDEN] = t0 * (E1P * v2 + E2P * vvc1 + E3P * vvc2 + w2 * (E2P + E3P));
    fm[UEDEN] = t0 * (E1M * v2 + E2M * vvc1 + E3M * vvc2 + w2 * (E2M + E3M));
}

// WENO-Z, Source/kernel/Reconstruction.H:83-138: f+ stencil at cells i-3..i+1
__host__ __device__ __forceinline__ double wenoz_plus(double V1, double V2, double V3, double V4, double V5) {
    const double eps = 1e-6;
    double s11 = (13.0 / 12.0) * (V1 - 2.0 * V2 + V3) * (V1 - 2.0 * V2 + V3) +
                 0.25 * (V1 - 4.0 * V2 + 3.0 * V3) * (V1 - 4.0 * V2 + 3.0 * V3);
    double s22 = (13.0 / 12.0) * (V2 - 2.0 * V3 + V4) * (V2 - 2.0 * V3 + V4) + 0.25 * (V2 - V4) * (V2 - V4);
    double s33 = (13.0 / 12.0) * (V3 - 2.0 * V4 + V5) * (V3 - 2.0 * V4 + V5) +
                 0.25 * (3.0 * V3 - 4.0 * V4 + V5) * (3.0 * V3 - 4.0 * V4 + V5);
    double s55 = fabs(s11 - s33);
    s11 = 1.0 + (s55 / (eps + s11)) * (s55 / (eps + s11));
    s22 = 1.0 + (s55 / (eps + s22)) * (s55 / (eps + s22));
    s33 = 1.0 + (s55 / (eps + s33)) * (s55 / (eps + s33));
    double a1 = s11, a2 = 6.0 * s22, a3 = 3.0 * s33;
    double invsum = 1.0 / (a1 + a2 + a3);
    double v1 = 2.0 * V1 - 7.0 * V2 + 11.0 * V3;
    double v2 = -V2 + 5.0 * V3 + 2.0 * V4;
    double v3 = 2.0 * V3 + 5.0 * V4 - V5;
    return (1.0 / 6.0) * invsum * (a1 * v1 + a2 * v2 + a3 * v3);
}

// ... and the mirrored f- stencil at cells i-2..i+2
__host__ __device__ __forceinline__ double wenoz_minus(double V1, double V2, double V3, double V4, double V5) {
    const double eps = 1e-6;
    double s11 = (13.0 / 12.0) * (V5 - 2.0 * V4 + V3) * (V5 - 2.0 * V4 + V3) +
                 0.25 * (V5 - 4.0 * V4 + 3.0 * V3) * (V5 - 4.0 * V4 + 3.0 * V3);
    double s22 = (13.0 / 12.0) * (V2 - 2.0 * V3 + V4) * (V2 - 2.0 * V3 + V4) + 0.25 * (V4 - V2) * (V4 - V2);
    double s33 = (13.0 / 12.0) * (V3 - 2.0 * V2 + V1) * (V3 - 2.0 * V2 + V1) +
                 0.25 * (3.0 * V3 - 4.0 * V2 + V1) * (3.0 * V3 - 4.0 * V2 + V1);
    double s55 = fabs(s11 - s33);
    s11 = 1.0 + (s55 / (eps + s11)) * (s55 / (eps + s11));
    s22 = 1.0 + (s55 / (eps + s22)) * (s55 / (eps + s22));
    s33 = 1.0 + (s55 / (eps + s33)) * (s55 / (eps + s33));
    double a1 = s11, a2 = 6.0 * s22, a3 = 3.0 * s33;
    double invsum = 1.0 / (a1 + a2 + a3);
    double v1 = 11.0 * V3 - 7.0 * V4 + 2.0 * V5;
    double v2 = -V4 + 5.0 * V3 + 2.0 * V2;
    double v3 = 2.0 * V3 + 5.0 * V2 - V1;
    return (1.0 / 6.0) * invsum * (a1 * v1 + a2 * v2 + a3 * v3);
}

#if defined(__CUDACC__)
// 1/x for a normal, finite, non-zero double, to within about one ulp, without an
// IEEE division: the PTX approximate reciprocal (rcp.approx.ftz.f64, a seed
// good to roughly 20 bits) refined by two Newton-Raphson steps
// r <- r + r (1 - x r), each of which squares the relative error (P. Markstein,
// IBM J. Res. Develop. 34 (1990) 111-119).  GB300 issues few FP64 instructions
// per cycle; this takes one MUFU operation and four FMAs where a correctly
// rounded division takes about twice as many FP64 instructions.  The
// arguments it is used on are sums of squares plus a positive epsilon.
__device__ __forceinline__ double rcp_nr(double x) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    double e = fma(-x, r, 1.0);
    r = fma(r, e, r);
    e = fma(-x, r, 1.0);
    return fma(r, e, r);
}

// WENO-Z of one split flux (Source/kernel/Reconstruction.H:83-138) with a
// single reciprocal in place of the reference's four divisions, in the
// fewest FP64 operations (GB300 issues two FP64 instructions per cycle per SM).
// The stencil V1..V5 is ordered towards the face (f+: cells i-3..i+1; f-:
// cells i+2..i-2, i.e. wenoz_minus(V1..V5) == wenoz_1rcp(V5, V4, V3, V2, V1)).
//   - The smoothness indicators are carried as 4 beta_k = (13/3) e_k^2 + g_k^2
//     (e, g the second and first differences of the reference's beta_k), with
//     eps -> 4 eps: tau / (eps + beta_k) is unchanged, and the scaling by 4 is
//     exact.
//   - The weights alpha_k = d_k (1 + (tau / D_k)^2), D_k = eps + beta_k,
//     d = (1, 6, 3), are multiplied by the common positive factor
//     (D_1 D_2 D_3)^2, which cancels in alpha_k / sum alpha: with q_k = D_k^2
//     and P = q_1 q_2 q_3, alpha_k becomes d_k A_k, A_k = P + tau^2 q_j q_l
//     ({j, l} the other two).
//   - The face value sum_k alpha_k v_k / (6 sum_k alpha_k), v_k the candidate
//     polynomials (2, -7, 11), (-1, 5, 2), (2, 5, -1), is formed as
//     (A_1 v_1 / 6 + A_2 v_2 + A_3 v_3 / 2) / (A_1 + 6 A_2 + 3 A_3), the 1/6 and
//     the d_k folded into the polynomials' coefficients.
// The same value up to rounding (parity tests: 1e-12 per right-hand side); the
// products stay finite for |beta| < 2e50, i.e. flux differences below ~1e25.
//
// The second differences' (13/3) e^2 belong to a cell triple, and a triple
// serves as stencil 1, 2 and 3 of three consecutive faces: wenoz_run3 forms
// five of them for a run of three faces instead of nine.
__device__ __forceinline__ double wenoz_e2(double Va, double Vb, double Vc) {
    const double e = __dadd_rn(__fma_rn(-2.0, Vb, Va), Vc);
    return __dmul_rn(__dmul_rn(13.0 / 3.0, e), e);
}
// one side's face from its stencil V1..V5 (ordered towards the face) and the
// (13/3) e^2 of its triples (V1 V2 V3), (V2 V3 V4), (V3 V4 V5); every rounding
// written out, so the value does not depend on the code around the call
__device__ __forceinline__ double wenoz_face_e(double V1, double V2, double V3, double V4, double V5, double E1,
                                               double E2, double E3) {
    const double eps4 = 4e-6;
    const double g1 = __fma_rn(3.0, V3, __fma_rn(-4.0, V2, V1));
    const double g2 = __dsub_rn(V2, V4);
    const double g3 = __fma_rn(-4.0, V4, __fma_rn(3.0, V3, V5));
    const double b1 = __fma_rn(g1, g1, E1), b2 = __fma_rn(g2, g2, E2), b3 = __fma_rn(g3, g3, E3);
    const double tau = fabs(__dsub_rn(b1, b3));
    const double D1 = __dadd_rn(eps4, b1), D2 = __dadd_rn(eps4, b2), D3 = __dadd_rn(eps4, b3);
    const double q1 = __dmul_rn(D1, D1), q2 = __dmul_rn(D2, D2), q3 = __dmul_rn(D3, D3), t2 = __dmul_rn(tau, tau);
    const double q12 = __dmul_rn(q1, q2), q13 = __dmul_rn(q1, q3), q23 = __dmul_rn(q2, q3);
    const double Pq = __dmul_rn(q12, q3);
    const double A1 = __fma_rn(t2, q23, Pq), A2 = __fma_rn(t2, q13, Pq), A3 = __fma_rn(t2, q12, Pq);
    const double c1 = __fma_rn(11.0 / 6.0, V3, __fma_rn(-7.0 / 6.0, V2, __dmul_rn(1.0 / 3.0, V1)));
    const double c2 = __fma_rn(2.0, V4, __fma_rn(5.0, V3, -V2));
    const double c3 = __fma_rn(-0.5, V5, __fma_rn(2.5, V4, V3));
    const double num = __fma_rn(A3, c3, __fma_rn(A2, c2, __dmul_rn(A1, c1)));
    const double den = __fma_rn(3.0, A3, __fma_rn(6.0, A2, A1));
    return __dmul_rn(num, rcp_nr(den));
}
__device__ __forceinline__ double wenoz_1rcp(double V1, double V2, double V3, double V4, double V5) {
    return wenoz_face_e(V1, V2, V3, V4, V5, wenoz_e2(V1, V2, V3), wenoz_e2(V2, V3, V4), wenoz_e2(V3, V4, V5));
}
// one side of faces m = 0, 1, 2 whose stencils (ordered towards the face) are
// a[m s] .. a[(m + 4) s], as a window sliding along the line (five values and
// three (13/3) e^2 live at a time).  The f+ side of a run is a = f+ at the
// first face's stencil start, s = the pencil stride; its f- side is a = f- at
// (start + 7 s), s = -stride, and yields the faces in reverse order.
__device__ __forceinline__ void wenoz_run3(const double* a, int s, double& o0, double& o1, double& o2) {
    double A0 = a[0], A1 = a[s], A2 = a[2 * s], A3 = a[3 * s], A4 = a[4 * s];
    double E0 = wenoz_e2(A0, A1, A2), E1 = wenoz_e2(A1, A2, A3), E2 = wenoz_e2(A2, A3, A4);
#pragma unroll 1
    for (int m = 0; m < 3; ++m) {
        const double v = wenoz_face_e(A0, A1, A2, A3, A4, E0, E1, E2);
        if (m == 0) o0 = v;
        else if (m == 1) o1 = v;
        else o2 = v;
        if (m < 2) {
            A0 = A1;
            A1 = A2;
            A2 = A3;
            A3 = A4;
            A4 = a[(m + 5) * s];
            E0 = E1;
            E1 = E2;
            E2 = wenoz_e2(A2, A3, A4);
        }
    }
}
#endif

#if defined(__CUDACC__)
// The positive and negative parts the reference forms as (x + |x|)/2 and
// x - (x + |x|)/2 (FluxSplit.H:46-51) are exactly x or +0 (and -0 for the
// negative part of -0): selected on the sign bit, on the integer pipes.
__device__ __forceinline__ double pos_part(double x) { return __double_as_longlong(x) > 0 ? x : 0.0; }
__device__ __forceinline__ double neg_part(double x) { return __double_as_longlong(x) < 0 ? x : 0.0; }

// Steger-Warming split along D (Source/kernel/FluxSplit.H:11-193) for the fused
// FP64 kernels, in fewer FP64 operations than sw_split's reference order: with
// un the normal and ua, ub the tangential velocities, qt = ua^2 + ub^2 is shared
// by the three |.|^2 terms, the energy flux's E2 vvc1 + E3 vvc2 + w2 (E2 + E3)
// is E2 (vvc1 + w2) + E3 (vvc2 + w2), and the tangential momentum fluxes are
// the mass flux times the velocity.  The eigenvalue parts are exact selects.
// The same values up to rounding (parity tests: 1e-12 per right-hand side);
// every rounding is written out, so the fluxes of a cell do not depend on the
// code around the call.
template <int D>
__device__ __forceinline__ void sw_split_d(double d, double u, double v, double w, double c, double t1, double t2,
                                           double t3, double gm1, double* fp, double* fm) {
    const double vel[3] = {u, v, w};
    const double un = vel[D], ua = vel[(D + 1) % 3], ub = vel[(D + 2) % 3];
    const double qt = __fma_rn(ub, ub, __dmul_rn(ua, ua));
    const double uc1 = __dsub_rn(un, c), uc2 = __dadd_rn(un, c);
    const double w2 = __dmul_rn(__dmul_rn(t3, c), c);
    const double v2 = __dmul_rn(gm1, __fma_rn(un, un, qt));
    const double h1 = __fma_rn(0.5, __fma_rn(uc1, uc1, qt), w2);  // vvc1 + w2
    const double h2 = __fma_rn(0.5, __fma_rn(uc2, uc2, qt), w2);  // vvc2 + w2
    const double E1P = pos_part(un), E2P = pos_part(uc1), E3P = pos_part(uc2);
    const double E1M = neg_part(un), E2M = neg_part(uc1), E3M = neg_part(uc2);
    const double t0 = __dmul_rn(d, t1);
    const double a1p = __dmul_rn(t2, E1P), a1m = __dmul_rn(t2, E1M);
    const double rp = __dmul_rn(t0, __dadd_rn(__dadd_rn(a1p, E2P), E3P));
    const double rm = __dmul_rn(t0, __dadd_rn(__dadd_rn(a1m, E2M), E3M));
    fp[URHO] = rp;
    fm[URHO] = rm;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        if (m == D) {
            fp[UMX + m] = __dmul_rn(t0, __fma_rn(E3P, uc2, __fma_rn(E2P, uc1, __dmul_rn(a1p, un))));
            fm[UMX + m] = __dmul_rn(t0, __fma_rn(E3M, uc2, __fma_rn(E2M, uc1, __dmul_rn(a1m, un))));
        } else {
            fp[UMX + m] = __dmul_rn(rp, vel[m]);
            fm[UMX + m] = __dmul_rn(rm, vel[m]);
        }
    }
    fp[UEDEN] = __dmul_rn(t0, __fma_rn(E3P, h2, __fma_rn(E2P, h1, __dmul_rn(E1P, v2))));
    fm[UEDEN] = __dmul_rn(t0, __fma_rn(E3M, h2, __fma_rn(E2M, h1, __dmul_rn(E1M, v2))));
}
#endif

#if defined(__CUDACC__)
// max(a, b) for b > 0 (the density and pressure floors) on the integer pipes:
// a double's bits read as a signed integer order as the double does against a
// positive b, a negative a or -0 reading below it (NaN a is the only case that
// differs from a > b ? a : b)
__device__ __forceinline__ double max_floor(double a, double b) {
    return __double_as_longlong(a) > __double_as_longlong(b) ? a : b;
}

// c2prim (Source/kernel/Kernels.H:13-40) for the fused FP64 kernels, in fewer
// FP64 operations: the two divisions become one reciprocal of rho
// (T = p (1/rho) (1/Rg), 1/Rg formed once on the host), the floors are integer
// compares, rho |u|^2 is formed as the momenta times the velocities, and
// c^2 = gamma Rg T as gamma p (1/rho); the same values to within a few ulps.
__device__ __forceinline__ void c2prim_ideal_fast(const DevParm& P, double u0, double u1, double u2, double u3,
                                                  double u4, double* q) {
    const double rho = max_floor(u0, P.smallr);
    const double rhoinv = rcp_nr(rho);
    const double ux = u1 * rhoinv, uy = u2 * rhoinv, uz = u3 * rhoinv;
    const double ei = fma(-0.5, fma(u3, uz, fma(u2, uy, u1 * ux)), u4);
    const double p = max_floor((P.gamma - 1.0) * ei, P.smallp);
    q[QRHO] = rho;
    q[QU] = ux;
    q[QV] = uy;
    q[QW] = uz;
    q[QPRES] = p;
    q[QT] = p * rhoinv * P.invRg;
    q[QC] = sqrt(P.gamma * p * rhoinv);
}
#endif

__host__ __device__ __forceinline__ double sutherland(const DevParm& P, double T) {
    return P.C_s * T * sqrt(T) / (T + P.T_s);
}

}  // namespace ocfd
