/* Source-compatible per-point functions of OpenCFD-AMR's ideal-gas kernel headers.
 *
 * The reference's regular-box chain (Source/Advance.cpp:245-329) calls, inside
 * amrex::ParallelFor lambdas,
 *   c2prim            Source/kernel/Kernels.H:13-40
 *   flux_split_x/y/z  Source/kernel/FluxSplit.H:11-193
 *   reconstruction_x/y/z (WENO-Z)  Source/kernel/Reconstruction.H:70-279
 *   compute_visc_x/y/z  Source/kernel/Diffusion.H:7-131
 *   divop             Source/kernel/Kernels.H:84-97
 * This header provides the same names with the same arguments and results,
 * computed by this library's point arithmetic (the functions the fused GPU
 * kernels are built from), so that Advance.cpp can include it in place of those
 * headers and keep its per-point loops unchanged.  The fused per-box entry
 * points of ocfd.h are the fast path; these are the drop-in for a build that
 * keeps the reference's structure.
 *
 * Array arguments: any type with operator()(i, j, k, n) returning a reference
 * (amrex::Array4<Real> / Array4<Real const>); dxinv: any type with operator[]
 * (amrex::GpuArray<Real, 3>); parm: the reference's Parm or ocfd_parm (members
 * eos_gamma, Rg, smallr, smallp, C_s, T_s, kOverMu, twoThirds).  Ideal gas
 * (the CHEM build's gamma-per-cell split is not covered here: the multispecies
 * chain is reached through ocfd_rhs_chem_box_f64).  Compile with nvcc. */
#ifndef OCFD_COMPAT_H
#define OCFD_COMPAT_H

#include "../../opencfd-amr_gb300/csrc/device_physics.cuh"

namespace ocfd_compat {

template <class P>
__host__ __device__ __forceinline__ ocfd::DevParm point_parm(const P& parm) {
    ocfd::DevParm d{};
    d.gamma = parm.eos_gamma;
    d.Rg = parm.Rg;
    d.smallr = parm.smallr;
    d.smallp = parm.smallp;
    d.C_s = parm.C_s;
    d.T_s = parm.T_s;
    d.kOverMu = parm.kOverMu;
    d.twoThirds = parm.twoThirds;
    return d;
}

// q = rho, u, v, w, p, T, c from the conserved state
template <class U, class Q, class P>
__host__ __device__ __forceinline__ void c2prim(int i, int j, int k, const U& u, const Q& q, const P& parm) noexcept {
    double w[7];
    ocfd::c2prim_ideal(point_parm(parm), u(i, j, k, 0), u(i, j, k, 1), u(i, j, k, 2), u(i, j, k, 3), u(i, j, k, 4),
                       w);
    for (int m = 0; m < 7; ++m) q(i, j, k, m) = w[m];
}

// Steger-Warming F+ / F- of cell (i, j, k) along D
template <int D, class F, class Q, class P>
__host__ __device__ __forceinline__ void flux_split(int i, int j, int k, const F& fp, const F& fm, const Q& q,
                                                   const P& parm) noexcept {
    const double g = parm.eos_gamma;
    const double t1 = 1.0 / (2.0 * g), t2 = 2.0 * (g - 1.0), t3 = (3.0 - g) / (2.0 * (g - 1.0));
    double a[5], b[5];
    ocfd::sw_split<D, double>(q(i, j, k, ocfd::QRHO), q(i, j, k, ocfd::QU), q(i, j, k, ocfd::QV),
                              q(i, j, k, ocfd::QW), q(i, j, k, ocfd::QC), t1, t2, t3, g - 1, a, b);
    for (int n = 0; n < 5; ++n) {
        fp(i, j, k, n) = a[n];
        fm(i, j, k, n) = b[n];
    }
}

template <class F, class Q, class S, class P>
__host__ __device__ __forceinline__ void flux_split_x(int i, int j, int k, const F& fp, const F& fm, const Q& q,
                                                     const S& /*state*/, const P& parm) noexcept {
    flux_split<0>(i, j, k, fp, fm, q, parm);
}
template <class F, class Q, class S, class P>
__host__ __device__ __forceinline__ void flux_split_y(int i, int j, int k, const F& fp, const F& fm, const Q& q,
                                                     const S& /*state*/, const P& parm) noexcept {
    flux_split<1>(i, j, k, fp, fm, q, parm);
}
template <class F, class Q, class S, class P>
__host__ __device__ __forceinline__ void flux_split_z(int i, int j, int k, const F& fp, const F& fm, const Q& q,
                                                     const S& /*state*/, const P& parm) noexcept {
    flux_split<2>(i, j, k, fp, fm, q, parm);
}

// WENO-Z face flux of component n on the D-face between cells (i,j,k) - e_D and
// (i,j,k): F+ from the cells i-3..i+1, F- from i-2..i+2 (along D)
template <int D, class F, class X>
__host__ __device__ __forceinline__ void reconstruction(int i, int j, int k, int n, const F& fp, const F& fm,
                                                       const X& flux) noexcept {
    const int di = D == 0, dj = D == 1, dk = D == 2;
    auto at = [&](const F& a, int s) { return a(i + s * di, j + s * dj, k + s * dk, n); };
    flux(i, j, k, n) = ocfd::wenoz_plus(at(fp, -3), at(fp, -2), at(fp, -1), at(fp, 0), at(fp, 1)) +
                       ocfd::wenoz_minus(at(fm, -2), at(fm, -1), at(fm, 0), at(fm, 1), at(fm, 2));
}

template <class F, class X, class P>
__host__ __device__ __forceinline__ void reconstruction_x(int i, int j, int k, int n, const F& fp, const F& fm,
                                                         const X& fxfab, const P& /*parm*/) noexcept {
    reconstruction<0>(i, j, k, n, fp, fm, fxfab);
}
template <class F, class X, class P>
__host__ __device__ __forceinline__ void reconstruction_y(int i, int j, int k, int n, const F& fp, const F& fm,
                                                         const X& fyfab, const P& /*parm*/) noexcept {
    reconstruction<1>(i, j, k, n, fp, fm, fyfab);
}
template <class F, class X, class P>
__host__ __device__ __forceinline__ void reconstruction_z(int i, int j, int k, int n, const F& fp, const F& fm,
                                                         const X& fzfab, const P& /*parm*/) noexcept {
    reconstruction<2>(i, j, k, n, fp, fm, fzfab);
}

// Viscous stress and heat flux subtracted from the D-face flux: Sutherland
// viscosity of the two cells, k = mu kOverMu, the normal derivatives across the
// face and the transverse ones averaged over the face's two cells
template <int D, class Q, class X, class A, class P>
__host__ __device__ __forceinline__ void compute_visc(int i, int j, int k, const Q& q, const X& f, const A& dxinv,
                                                     const P& parm) noexcept {
    const ocfd::DevParm pp = point_parm(parm);
    const int e[3] = {D == 0, D == 1, D == 2};
    const int il = i - e[0], jl = j - e[1], kl = k - e[2];
    const double Tr = q(i, j, k, ocfd::QT), Tl = q(il, jl, kl, ocfd::QT);
    const double mutl = ocfd::sutherland(pp, Tl), mutr = ocfd::sutherland(pp, Tr);
    const double ktl = mutl * parm.kOverMu, ktr = mutr * parm.kOverMu;
    const double dT = (Tr - Tl) * dxinv[D];
    double g[3][3];  // g[m][t] = d(u_m)/dx_t at the face
    for (int m = 0; m < 3; ++m) g[m][D] = (q(i, j, k, ocfd::QU + m) - q(il, jl, kl, ocfd::QU + m)) * dxinv[D];
    for (int t = 0; t < 3; ++t) {
        if (t == D) continue;
        const int a = t == 0, b = t == 1, c = t == 2;
        const int m2[2] = {D, t};
        for (int w = 0; w < 2; ++w) {
            const int m = ocfd::QU + m2[w];
            g[m2[w]][t] = (q(i + a, j + b, k + c, m) + q(il + a, jl + b, kl + c, m) - q(i - a, j - b, k - c, m) -
                           q(il - a, jl - b, kl - c, m)) *
                          (0.25 * dxinv[t]);
        }
    }
    const double divu = g[0][0] + g[1][1] + g[2][2];
    const double muf = 0.5 * (mutl + mutr);
    double tau[3];
    for (int m = 0; m < 3; ++m)
        tau[m] = (m == D) ? muf * (2.0 * g[D][D] - parm.twoThirds * divu) : muf * (g[m][D] + g[D][m]);
    for (int m = 0; m < 3; ++m) f(i, j, k, 1 + m) += -tau[m];
    f(i, j, k, 4) += -0.5 * ((q(i, j, k, ocfd::QU) + q(il, jl, kl, ocfd::QU)) * tau[0] +
                             (q(i, j, k, ocfd::QV) + q(il, jl, kl, ocfd::QV)) * tau[1] +
                             (q(i, j, k, ocfd::QW) + q(il, jl, kl, ocfd::QW)) * tau[2] + (ktl + ktr) * dT);
}

template <class Q, class X, class A, class P>
__host__ __device__ __forceinline__ void compute_visc_x(int i, int j, int k, const Q& q, const X& fx, const A& dxinv,
                                                       const P& parm) noexcept {
    compute_visc<0>(i, j, k, q, fx, dxinv, parm);
}
template <class Q, class X, class A, class P>
__host__ __device__ __forceinline__ void compute_visc_y(int i, int j, int k, const Q& q, const X& fy, const A& dxinv,
                                                       const P& parm) noexcept {
    compute_visc<1>(i, j, k, q, fy, dxinv, parm);
}
template <class Q, class X, class A, class P>
__host__ __device__ __forceinline__ void compute_visc_z(int i, int j, int k, const Q& q, const X& fz, const A& dxinv,
                                                       const P& parm) noexcept {
    compute_visc<2>(i, j, k, q, fz, dxinv, parm);
}

// dS/dt of component n: sum over x, y, z (in that order) of dxinv_d (F_d(i) - F_d(i + e_d))
template <class X, class F, class A>
__host__ __device__ __forceinline__ void divop(int i, int j, int k, int n, const X& dudt, const F& fx, const F& fy,
                                              const F& fz, const A& dxinv) noexcept {
    dudt(i, j, k, n) = dxinv[0] * (fx(i, j, k, n) - fx(i + 1, j, k, n)) +
                       dxinv[1] * (fy(i, j, k, n) - fy(i, j + 1, k, n)) +
                       dxinv[2] * (fz(i, j, k, n) - fz(i, j, k + 1, n));
}

}  // namespace ocfd_compat

#endif
