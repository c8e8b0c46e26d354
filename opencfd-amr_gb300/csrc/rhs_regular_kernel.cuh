// Fused regular-box right-hand side, templated on the precision of the flux
// evaluation FT:
//   FT = double  the plain FP64 form (reference operation order; parity 1e-12)
//   FT = float   the mixed-precision form: primitives, Steger-Warming split,
//                WENO-Z (stencils normalised by a power of two, the smoothness
//                epsilon rescaled into the normalised units), viscous flux and
//                divergence in FP32, state narrowed / divergence widened on the
//                integer pipes; the RK accumulation stays FP64 (the CFL bound
//                of the new state is evaluated in FP32).
// Included by rhs_regular.cu (double) and rhs_regular_f32.cu (float).
//
// One CTA owns a TX x TY x TZ tile.  Per direction D:
//   1. the tile's pencil along D (tile + 3 cells each side) is read from the
//      state, turned into primitives and split into F+ / F- (10 values per
//      cell) in shared memory,
//   2. WENO-Z face fluxes of the tile's T_D+1 faces x 5 components are formed
//      in shared memory (work items = face x component),
//   3. with OCFD_VISC the viscous stress / heat flux is added per face from a
//      primitive ring (tile grown by 1) staged once per tile,
//   4. each cell thread accumulates dxinv_D (F_f - F_f+1) in registers in the
//      reference's summation order x, y, z (Source/kernel/Kernels.H:94-96);
//      face fluxes are written out when the caller asked for them (reflux).
// Only U (read) and the output touch HBM.
//
// FP32-flux form on tiles of depth >= 4 (CrossOn): step 1 reads no global
// memory.  Before the sweeps, the tile's cross - its centre and the +-3 halos
// along x, y and z, every cell a pencil reads - is copied from the state FAB
// into shared memory by seven TMA box loads (cp.async.bulk.tensor, completing
// on an mbarrier with a bounded wait), narrowed and turned into primitives once
// per cell (Q), and each direction's pencil is split from Q.  The primitives of
// a cell are the same function of the same state either way, so the results
// are bit-identical to the pencil-by-pencil form.
// FP64 inviscid tiles (CrossPlain) keep the same cross of primitives in FP64,
// formed once per cell with plain loads (no TMA: one CTA per SM is resident, and
// its loads are the FP64 pipe's shadow), where the cross and the pencil region
// fit a CTA's shared memory.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>

#include "device_physics.cuh"
#include "weno_f32.cuh"
#include "ocfd_internal.h"
#include "rhs_regular.h"
#include "tma.cuh"

namespace ocfd {

constexpr size_t kMaxSmem = 227 * 1024;  // opt-in dynamic shared memory per CTA

template <int D, int TX, int TY, int TZ>
struct Pencil {
    static constexpr int PX = TX + (D == 0 ? 6 : 0);
    static constexpr int PY = TY + (D == 1 ? 6 : 0);
    static constexpr int PZ = TZ + (D == 2 ? 6 : 0);
    static constexpr int N = PX * PY * PZ;
    static constexpr int FX = TX + (D == 0);
    static constexpr int FY = TY + (D == 1);
    static constexpr int FZ = TZ + (D == 2);
    static constexpr int NF = FX * FY * FZ;
    static constexpr int PST = D == 0 ? 1 : (D == 1 ? PX : PX * PY);  // pencil stride along D
    static constexpr int FST = D == 0 ? 1 : (D == 1 ? FX : FX * FY);  // face stride along D
    static constexpr int SMEM = 10 * N + 5 * NF;                       // elements
};

template <int TX, int TY, int TZ>
struct Ring {
    static constexpr int RX = TX + 2, RY = TY + 2, RZ = TZ + 2;
    static constexpr int N = RX * RY * RZ;
};

template <int TX, int TY, int TZ>
__host__ __device__ constexpr int pencil_elems() {
    constexpr int a = Pencil<0, TX, TY, TZ>::SMEM;
    constexpr int b = Pencil<1, TX, TY, TZ>::SMEM;
    constexpr int c = Pencil<2, TX, TY, TZ>::SMEM;
    return a > b ? (a > c ? a : c) : (b > c ? b : c);
}

// tiles whose cross is staged by TMA (see the file comment): the staged
// variants (XS) of the tile shapes of depth >= 4 in the FP32-flux form
template <class FT, int TX, int TY, int TZ, bool VISC, bool XS>
struct CrossOn {
    static constexpr bool value = XS && std::is_same<FT, float>::value && !VISC && TZ >= 4 && TX % 2 == 0;
};

// Shared memory of a TMA-staged tile (offsets from a 128-byte aligned base):
//   region A  the FP64 staging boxes - centre TX x TY x TZ, x halos 4 x TY x TZ
//             (low one from 4 cells before the tile), y halos TX x 3 x TZ, z halos
//             TX x TY x 3, 5 components each, x fastest, each 128-byte aligned -
//             reused by the sweeps for the split and face fluxes;
//   Q         FP32 primitives rho, u, v, w, c of the cross, 5 planes of NQ cells:
//             centre, x halo (6 x TY x TZ: 3 low then 3 high), y halo
//             (TX x 6 x TZ), z halo (TX x TY x 6).
template <int TX, int TY, int TZ>
struct Cross {
    static constexpr int NC = TX * TY * TZ;
    static constexpr int NXH = 6 * TY * TZ, NYH = 6 * TX * TZ, NZH = 6 * TX * TY;
    static constexpr int NQ = NC + NXH + NYH + NZH;
    static constexpr int SX = 4 * TY * TZ, SY = 3 * TX * TZ, SZ = 3 * TX * TY;  // cells of one halo box
    static constexpr int al(int d) { return (d + 15) / 16 * 16; }              // doubles, to 128 bytes
    static constexpr int OC = 0, OXL = al(5 * NC), OXH = OXL + al(5 * SX), OYL = OXH + al(5 * SX),
                         OYH = OYL + al(5 * SY), OZL = OYH + al(5 * SY), OZH = OZL + al(5 * SZ),
                         NSTAGE = OZH + al(5 * SZ);
    static constexpr uint32_t BYTES_CXY = 8u * 5u * (NC + 2 * SX + 2 * SY), BYTES_Z = 8u * 5u * 2 * SZ;
    // Q index of tile-local (x, y, z) of a pencil along D: only the D coordinate
    // may lie outside the tile
    template <int D>
    __device__ static __forceinline__ int q_along(int x, int y, int z) {
        if (D == 0) {
            if (x < 0) return NC + (x + 3) + 6 * (y + TY * z);
            if (x >= TX) return NC + (x - TX + 3) + 6 * (y + TY * z);
        } else if (D == 1) {
            if (y < 0) return NC + NXH + x + TX * ((y + 3) + 6 * z);
            if (y >= TY) return NC + NXH + x + TX * ((y - TY + 3) + 6 * z);
        } else {
            if (z < 0) return NC + NXH + NYH + x + TX * (y + TY * (z + 3));
            if (z >= TZ) return NC + NXH + NYH + x + TX * (y + TY * (z - TZ + 3));
        }
        return x + TX * (y + TY * z);
    }
};

// FP64 inviscid tiles keep the same cross of primitives (layout Cross, FP64
// values) behind the pencil region, formed once per cell with plain loads, where
// the two fit a CTA's shared memory (one 512-thread CTA per SM: registers, not
// shared memory, bound the FP64 tiles)
template <int TX, int TY, int TZ>
__host__ __device__ constexpr size_t cross_plain_bytes() {
    return sizeof(double) * (pencil_elems<TX, TY, TZ>() + 5 * (size_t)Cross<TX, TY, TZ>::NQ);
}
template <class FT, int TX, int TY, int TZ, bool VISC>
struct CrossPlain {
    static constexpr bool value =
        std::is_same<FT, double>::value && !VISC && cross_plain_bytes<TX, TY, TZ>() <= kMaxSmem;
};

template <class FT, int TX, int TY, int TZ>
__host__ __device__ constexpr size_t cross_region_a() {
    const size_t st = 8 * (size_t)Cross<TX, TY, TZ>::NSTAGE;
    const size_t pe = (sizeof(FT) * pencil_elems<TX, TY, TZ>() + 127) / 128 * 128;
    return st > pe ? st : pe;
}

template <class FT, int TX, int TY, int TZ, bool VISC, bool XS = false>
__host__ __device__ constexpr size_t regular_smem_bytes() {
    if (CrossOn<FT, TX, TY, TZ, VISC, XS>::value)
        return 128 + cross_region_a<FT, TX, TY, TZ>() + sizeof(float) * 5 * Cross<TX, TY, TZ>::NQ;
    if (CrossPlain<FT, TX, TY, TZ, VISC>::value) return cross_plain_bytes<TX, TY, TZ>();
    return sizeof(FT) * (pencil_elems<TX, TY, TZ>() + (VISC ? 4 * Ring<TX, TY, TZ>::N : 0));
}

// ------------------------------------------------------------ precision traits
template <class FT>
struct Prec;

// FP64: the reference's expressions
template <>
struct Prec<double> {
    // q = rho, u, v, w, p, T, c
    static __device__ __forceinline__ void prims(const DevParm& P, const View<const double>& S, int i,
                                                 int j, int k, double* q) {
        c2prim_ideal_fast(P, S(i, j, k, 0), S(i, j, k, 1), S(i, j, k, 2), S(i, j, k, 3), S(i, j, k, 4), q);
    }
    template <int D>
    static __device__ __forceinline__ void split(const DevParm& P, const double* q, double* fp, double* fm) {
        sw_split_d<D>(q[QRHO], q[QU], q[QV], q[QW], q[QC], P.sw_tmp1, P.sw_tmp2, P.sw_tmp3, P.sw_gm1, fp, fm);
    }
    static __device__ __forceinline__ double weno(const double* a, const double* b, int s) {
        return wenoz_1rcp(a[0], a[s], a[2 * s], a[3 * s], a[4 * s]) +
               wenoz_1rcp(b[5 * s], b[4 * s], b[3 * s], b[2 * s], b[s]);
    }
    static __device__ __forceinline__ double mu(const DevParm& P, double T) { return sutherland(P, T); }
};

template <>
struct Prec<float> {
    // c2prim in FP32 from the narrowed conserved state
    static __device__ __forceinline__ void prims(const DevParm& P, const View<const double>& S, int i,
                                                 int j, int k, float* q) {
        prims_vals(P, S(i, j, k, 0), S(i, j, k, 1), S(i, j, k, 2), S(i, j, k, 3), S(i, j, k, 4), q);
    }
    static __device__ __forceinline__ void prims_vals(const DevParm& P, double s0, double s1, double s2, double s3,
                                                      double s4, float* q) {
        const float g = P.f_gamma;
        const float u0 = d2f_bits(s0), u1 = d2f_bits(s1), u2 = d2f_bits(s2), u3 = d2f_bits(s3), u4 = d2f_bits(s4);
        // every rounding written out (see sw_split_f32): the primitives do not
        // depend on the code around the call
        const float rho = fmaxf(u0, P.f_smallr);
        const float rhoinv = __frcp_rn(rho);
        const float ux = __fmul_rn(u1, rhoinv), uy = __fmul_rn(u2, rhoinv), uz = __fmul_rn(u3, rhoinv);
        const float ke = __fmaf_rn(uz, uz, __fmaf_rn(uy, uy, __fmul_rn(ux, ux)));
        const float ei = __fmaf_rn(-rho, __fmul_rn(0.5f, ke), u4);
        const float p = fmaxf(__fmul_rn(__fsub_rn(g, 1.0f), ei), P.f_smallp);
        q[QRHO] = rho;
        q[QU] = ux;
        q[QV] = uy;
        q[QW] = uz;
        q[QPRES] = p;
        q[QT] = __fmul_rn(__fmul_rn(p, rhoinv), P.f_invRg);
        q[QC] = __fsqrt_rn(__fmul_rn(__fmul_rn(g, p), rhoinv));
    }
    template <int D>
    static __device__ __forceinline__ void split(const DevParm& P, const float* q, float* fp, float* fm) {
        sw_split_f32<D>(q[QRHO], q[QU], q[QV], q[QW], q[QC], P.f_sw_tmp1, P.f_sw_tmp2, P.f_sw_tmp3, P.f_sw_gm1,
                        fp, fm);
    }
    static __device__ __forceinline__ float weno(const float* a, const float* b, int s) {
        return wenoz_pm_f(a[0], a[s], a[2 * s], a[3 * s], a[4 * s], b[5 * s], b[4 * s], b[3 * s], b[2 * s], b[s]);
    }
    static __device__ __forceinline__ float mu(const DevParm& P, float T) {
        return P.f_C_s * T * sqrtf(T) / (T + P.f_T_s);
    }
};

// Viscous stress and heat flux of the D-face between ring cells (r - e_D) and r,
// Source/kernel/Diffusion.H:7-131.  ring holds u, v, w, T (4 planes of RN).
// CFL bound of the new state (Source/Advance.cpp:26-49): FP64 in the plain form,
// FP32 (from the narrowed state) in the mixed form
template <class FT>
__device__ __forceinline__ double stage_cfl_bound(const DevParm& P, const double* un, const RegBoxArgs& B) {
    return cfl_bound(P, un, B.dx);
}
template <>
__device__ __forceinline__ double stage_cfl_bound<float>(const DevParm& P, const double* un, const RegBoxArgs& B) {
    const float g = P.f_gamma;
    const float rho = d2f_bits(un[0]);
    const float rhoinv = __frcp_rn(fmaxf(rho, P.f_smallr));
    // every rounding written out (see sw_split_f32)
    const float vx = __fmul_rn(d2f_bits(un[1]), rhoinv), vy = __fmul_rn(d2f_bits(un[2]), rhoinv),
                vz = __fmul_rn(d2f_bits(un[3]), rhoinv);
    const float ke = __fmaf_rn(vz, vz, __fmaf_rn(vy, vy, __fmul_rn(vx, vx)));
    const float p =
        fmaxf(__fmul_rn(__fsub_rn(g, 1.0f), __fmaf_rn(-__fmul_rn(0.5f, rho), ke, d2f_bits(un[4]))), P.f_smallp);
    const float cs = __fsqrt_rn(__fmul_rn(__fmul_rn(g, p), rhoinv));
    const float dtx = __fdividef(B.dx_f[0], __fadd_rn(fabsf(vx), cs));
    const float dty = __fdividef(B.dx_f[1], __fadd_rn(fabsf(vy), cs));
    const float dtz = __fdividef(B.dx_f[2], __fadd_rn(fabsf(vz), cs));
    return f2d_bits(fminf(dtx, fminf(dty, dtz)));
}

// box geometry and Parm constants in the flux precision
template <class FT>
__device__ __forceinline__ FT dxinv_of(const RegBoxArgs& B, int d) { return B.dxinv[d]; }
template <>
__device__ __forceinline__ float dxinv_of<float>(const RegBoxArgs& B, int d) { return B.dxinv_f[d]; }
template <class FT>
__device__ __forceinline__ FT kovermu_of(const DevParm& P) { return P.kOverMu; }
template <>
__device__ __forceinline__ float kovermu_of<float>(const DevParm& P) { return P.f_kOverMu; }
template <class FT>
__device__ __forceinline__ FT twothirds_of(const DevParm& P) { return P.twoThirds; }
template <>
__device__ __forceinline__ float twothirds_of<float>(const DevParm& P) { return P.f_twoThirds; }

template <class FT>
__device__ __forceinline__ double widen(FT x) { return (double)x; }
template <>
__device__ __forceinline__ double widen<float>(float x) { return f2d_bits(x); }

template <class FT, int D, int TX, int TY, int TZ>
__device__ __forceinline__ void visc_face(const DevParm& P, const FT* ring, int rx, int ry, int rz,
                                          const FT* dxinv, FT* f /*stride fs*/, int fs) {
    using R = Ring<TX, TY, TZ>;
    constexpr int S[3] = {1, R::RX, R::RX * R::RY};
    const FT kOverMu = kovermu_of<FT>(P), twoThirds = twothirds_of<FT>(P);
    const int c = rx + ry * R::RX + rz * R::RX * R::RY;
    const int l = c - S[D];
    const FT* qu = ring;
    const FT* qT = ring + 3 * R::N;
    const FT Tr = qT[c], Tl = qT[l];
    const FT mutl = Prec<FT>::mu(P, Tl), mutr = Prec<FT>::mu(P, Tr);
    const FT ktl = mutl * kOverMu, ktr = mutr * kOverMu;
    const FT dT = (Tr - Tl) * dxinv[D];
    FT g[3][3];
#pragma unroll
    for (int m = 0; m < 3; ++m) g[m][D] = (qu[m * R::N + c] - qu[m * R::N + l]) * dxinv[D];
#pragma unroll
    for (int t = 0; t < 3; ++t) {
        if (t == D) continue;
        const int st = S[t];
        // d(u_D)/dx_t and d(u_t)/dx_t averaged over the two cells of the face
        g[D][t] = (qu[D * R::N + c + st] + qu[D * R::N + l + st] - qu[D * R::N + c - st] -
                   qu[D * R::N + l - st]) * (FT(0.25) * dxinv[t]);
        g[t][t] = (qu[t * R::N + c + st] + qu[t * R::N + l + st] - qu[t * R::N + c - st] -
                   qu[t * R::N + l - st]) * (FT(0.25) * dxinv[t]);
    }
    const FT divu = g[0][0] + g[1][1] + g[2][2];
    const FT muf = FT(0.5) * (mutl + mutr);
    FT tau[3];
#pragma unroll
    for (int m = 0; m < 3; ++m)
        tau[m] = (m == D) ? muf * (FT(2.0) * g[D][D] - twoThirds * divu) : muf * (g[m][D] + g[D][m]);
#pragma unroll
    for (int m = 0; m < 3; ++m) f[(1 + m) * fs] += -tau[m];
    f[4 * fs] += FT(-0.5) * ((qu[c] + qu[l]) * tau[0] + (qu[R::N + c] + qu[R::N + l]) * tau[1] +
                             (qu[2 * R::N + c] + qu[2 * R::N + l]) * tau[2] + (ktl + ktr) * dT);
}

// Primitives of a TMA-staged tile's cross into Q (layout: Cross), once per cell:
// from the staged boxes, or with plain loads when the tile was not staged, for
// the z halo of a slab whose z ghosts are mirrored (zvirt: those boxes are not
// loaded) and for its cells outside the z domain.  Cells a pencil would not
// read (beyond hi + 3) are left 0; the sweeps never use them.
template <int TX, int TY, int TZ>
__device__ __forceinline__ void cross_prims(const RegBoxArgs& B, const DevParm& P, int i0, int j0, int k0,
                                            const double* stage, bool staged, float* Q) {
    using C = Cross<TX, TY, TZ>;
    constexpr int NT = TX * TY * TZ;
    for (int idx = threadIdx.x; idx < C::NQ; idx += NT) {
        int x, y, z, so, sc;
        bool zhalo = false;
        if (idx < C::NC) {
            x = idx % TX;
            y = (idx / TX) % TY;
            z = idx / (TX * TY);
            so = C::OC + idx;
            sc = C::NC;
        } else if (idx < C::NC + C::NXH) {
            const int r = idx - C::NC, h = r % 6;
            y = (r / 6) % TY;
            z = r / (6 * TY);
            x = h < 3 ? h - 3 : TX + h - 3;
            so = (h < 3 ? C::OXL + h + 1 : C::OXH + h - 3) + 4 * (y + TY * z);
            sc = C::SX;
        } else if (idx < C::NC + C::NXH + C::NYH) {
            const int r = idx - C::NC - C::NXH, h = (r / TX) % 6;
            x = r % TX;
            z = r / (6 * TX);
            y = h < 3 ? h - 3 : TY + h - 3;
            so = (h < 3 ? C::OYL + TX * h : C::OYH + TX * (h - 3)) + x + 3 * TX * z;
            sc = C::SY;
        } else {
            const int r = idx - C::NC - C::NXH - C::NYH, h = r / (TX * TY);
            x = r % TX;
            y = (r / TX) % TY;
            z = h < 3 ? h - 3 : TZ + h - 3;
            so = (h < 3 ? C::OZL + TX * TY * h : C::OZH + TX * TY * (h - 3)) + x + TX * y;
            sc = C::SZ;
            zhalo = true;
        }
        const int gi = i0 + x, gj = j0 + y, gk = k0 + z;
        float q[7] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        const bool zout = B.zvirt && (gk < B.zdom[0] || gk > B.zdom[1]);
        if (staged && !zout && !(zhalo && B.zvirt)) {
            Prec<float>::prims_vals(P, stage[so], stage[so + sc], stage[so + 2 * sc], stage[so + 3 * sc],
                                    stage[so + 4 * sc], q);
        } else if (gi <= B.hi[0] + 3 && gj <= B.hi[1] + 3 && (B.zvirt || gk <= B.hi[2] + 3)) {
            int sg;
            Prec<float>::prims(P, B.S, gi, gj, zmap(B, gk, sg), q);
            if (sg & 1) q[QU] = -q[QU];
            if (sg & 2) q[QV] = -q[QV];
            if (sg & 4) q[QW] = -q[QW];
        }
        Q[idx] = q[QRHO];
        Q[C::NQ + idx] = q[QU];
        Q[2 * C::NQ + idx] = q[QV];
        Q[3 * C::NQ + idx] = q[QW];
        Q[4 * C::NQ + idx] = q[QC];
    }
}

// Primitives of an FP64 tile's cross into Q (layout Cross, FP64 values), once
// per cell, with plain loads: the same cells, mirrored z ghosts and bounds as
// cross_prims (cells beyond hi + 3 are left 0; the sweeps never use them), and
// the same function of the state as the pencil-by-pencil form, so the sweeps
// give the same bits either way.
template <int TX, int TY, int TZ>
__device__ __forceinline__ void cross_prims_plain(const RegBoxArgs& B, const DevParm& P, int i0, int j0, int k0,
                                                  double* Q) {
    using C = Cross<TX, TY, TZ>;
    constexpr int NT = TX * TY * TZ;
    for (int idx = threadIdx.x; idx < C::NQ; idx += NT) {
        int x, y, z;
        if (idx < C::NC) {
            x = idx % TX;
            y = (idx / TX) % TY;
            z = idx / (TX * TY);
        } else if (idx < C::NC + C::NXH) {
            const int r = idx - C::NC, h = r % 6;
            y = (r / 6) % TY;
            z = r / (6 * TY);
            x = h < 3 ? h - 3 : TX + h - 3;
        } else if (idx < C::NC + C::NXH + C::NYH) {
            const int r = idx - C::NC - C::NXH, h = (r / TX) % 6;
            x = r % TX;
            z = r / (6 * TX);
            y = h < 3 ? h - 3 : TY + h - 3;
        } else {
            const int r = idx - C::NC - C::NXH - C::NYH, h = r / (TX * TY);
            x = r % TX;
            y = (r / TX) % TY;
            z = h < 3 ? h - 3 : TZ + h - 3;
        }
        const int gi = i0 + x, gj = j0 + y, gk = k0 + z;
        double q[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        if (gi <= B.hi[0] + 3 && gj <= B.hi[1] + 3 && (B.zvirt || gk <= B.hi[2] + 3)) {
            int sg;
            Prec<double>::prims(P, B.S, gi, gj, zmap(B, gk, sg), q);
            if (sg & 1) q[QU] = -q[QU];
            if (sg & 2) q[QV] = -q[QV];
            if (sg & 4) q[QW] = -q[QW];
        }
        Q[idx] = q[QRHO];
        Q[C::NQ + idx] = q[QU];
        Q[2 * C::NQ + idx] = q[QV];
        Q[3 * C::NQ + idx] = q[QW];
        Q[4 * C::NQ + idx] = q[QC];
    }
}

template <class FT, int D, int TX, int TY, int TZ, bool VISC, bool CROSS = false>
__device__ __forceinline__ void sweep(const RegBoxArgs& B, const DevParm& P, int i0, int j0, int k0,
                                      FT* F, FT* FF, const FT* ring, FT* acc, const FT* Q = nullptr) {
    using PC = Pencil<D, TX, TY, TZ>;
    constexpr int NT = TX * TY * TZ;
    const int tid = threadIdx.x;
    // ---- 1. primitives and Steger-Warming split over the pencil (primitives
    // from Q when the cross was staged)
    if constexpr (CROSS) {
        using C = Cross<TX, TY, TZ>;
        for (int c = tid; c < PC::N; c += NT) {
            const int px = c % PC::PX, py = (c / PC::PX) % PC::PY, pz = c / (PC::PX * PC::PY);
            const int lx = px - (D == 0 ? 3 : 0), ly = py - (D == 1 ? 3 : 0), lz = pz - (D == 2 ? 3 : 0);
            FT fp[5] = {0, 0, 0, 0, 0}, fm[5] = {0, 0, 0, 0, 0};
            if (i0 + lx <= B.hi[0] + (D == 0 ? 3 : 0) && j0 + ly <= B.hi[1] + (D == 1 ? 3 : 0) &&
                k0 + lz <= B.hi[2] + (D == 2 ? 3 : 0)) {
                const int qi = C::template q_along<D>(lx, ly, lz);
                FT q[7];
                q[QRHO] = Q[qi];
                q[QU] = Q[C::NQ + qi];
                q[QV] = Q[2 * C::NQ + qi];
                q[QW] = Q[3 * C::NQ + qi];
                q[QC] = Q[4 * C::NQ + qi];
                Prec<FT>::template split<D>(P, q, fp, fm);
            }
#pragma unroll
            for (int n = 0; n < 5; ++n) {
                F[n * PC::N + c] = fp[n];
                F[(5 + n) * PC::N + c] = fm[n];
            }
        }
    } else
    for (int c = tid; c < PC::N; c += NT) {
        const int px = c % PC::PX, py = (c / PC::PX) % PC::PY, pz = c / (PC::PX * PC::PY);
        const int gi = i0 + px - (D == 0 ? 3 : 0);
        const int gj = j0 + py - (D == 1 ? 3 : 0);
        const int gk = k0 + pz - (D == 2 ? 3 : 0);
        FT fp[5] = {0, 0, 0, 0, 0}, fm[5] = {0, 0, 0, 0, 0};
        if (gi <= B.hi[0] + (D == 0 ? 3 : 0) && gj <= B.hi[1] + (D == 1 ? 3 : 0) &&
            gk <= B.hi[2] + (D == 2 ? 3 : 0)) {
            FT q[7];
            int sg;
            const int gks = D == 2 ? zmap(B, gk, sg) : (sg = 0, gk);
            Prec<FT>::prims(P, B.S, gi, gj, gks, q);
            if (sg & 1) q[QU] = -q[QU];
            if (sg & 2) q[QV] = -q[QV];
            if (sg & 4) q[QW] = -q[QW];
            Prec<FT>::template split<D>(P, q, fp, fm);
        }
#pragma unroll
        for (int n = 0; n < 5; ++n) {
            F[n * PC::N + c] = fp[n];
            F[(5 + n) * PC::N + c] = fm[n];
        }
    }
    __syncthreads();
    // ---- 2. WENO-Z face fluxes
    if constexpr (std::is_same<FT, double>::value) {
        // FP64: a work item is a run of three consecutive faces of a line along
        // D (component n); runs start every three faces, the last one at FD - 3
        // so that every stencil stays in the pencil, and a run writes only the
        // faces from its own start on
        constexpr int FD = D == 0 ? PC::FX : (D == 1 ? PC::FY : PC::FZ);
        constexpr int NLINE = PC::NF / FD, NRUN = (FD + 2) / 3;
        static_assert(FD >= 3, "runs of three faces");
        for (int it = tid; it < 5 * NLINE * NRUN; it += NT) {
            const int n = it / (NLINE * NRUN), r = it - n * (NLINE * NRUN);
            const int line = r / NRUN, run = r - line * NRUN;
            const int fw = 3 * run, f0 = fw < FD - 3 ? fw : FD - 3;
            int fx, fy, fz;
            if (D == 0) {
                fx = f0; fy = line % PC::FY; fz = line / PC::FY;
            } else if (D == 1) {
                fx = line % PC::FX; fy = f0; fz = line / PC::FX;
            } else {
                fx = line % PC::FX; fy = line / PC::FX; fz = f0;
            }
            const int f = fx + fy * PC::FX + fz * PC::FX * PC::FY;
            const int base = fx + fy * PC::PX + fz * PC::PX * PC::PY;
            // f+ then f- (one side's registers at a time); the face flux is
            // f+ + f- as in the reference
            // f+ (side 0) then f- (side 1, faces in reverse order), one side's
            // window live at a time; the face flux is f+ + f-
            double p0 = 0.0, p1 = 0.0, p2 = 0.0;
            FT* out = FF + n * PC::NF + f;
#pragma unroll 1
            for (int side = 0; side < 2; ++side) {
                const double* a = side == 0 ? F + n * PC::N + base : F + (5 + n) * PC::N + base + 7 * PC::PST;
                const int st = side == 0 ? PC::PST : -PC::PST;
                double o0, o1, o2;
                wenoz_run3(a, st, o0, o1, o2);
                if (side == 0) {
                    p0 = o0;
                    p1 = o1;
                    p2 = o2;
                } else {
                    if (f0 >= fw) out[0] = __dadd_rn(p0, o2);
                    if (f0 + 1 >= fw) out[PC::FST] = __dadd_rn(p1, o1);
                    out[2 * PC::FST] = __dadd_rn(p2, o0);
                }
            }
        }
    } else {
        for (int it = tid; it < 5 * PC::NF; it += NT) {
            const int n = it / PC::NF, f = it - n * PC::NF;
            const int fx = f % PC::FX, fy = (f / PC::FX) % PC::FY, fz = f / (PC::FX * PC::FY);
            const int base = fx + fy * PC::PX + fz * PC::PX * PC::PY;
            FF[n * PC::NF + f] = Prec<FT>::weno(F + n * PC::N + base, F + (5 + n) * PC::N + base, PC::PST);
        }
    }
    __syncthreads();
    // ---- 3. viscous part of the face flux
    if (VISC) {
        const FT dxinvT[3] = {dxinv_of<FT>(B, 0), dxinv_of<FT>(B, 1), dxinv_of<FT>(B, 2)};
        for (int f = tid; f < PC::NF; f += NT) {
            const int fx = f % PC::FX, fy = (f / PC::FX) % PC::FY, fz = f / (PC::FX * PC::FY);
            // ring coordinates of the cell on the high side of the face
            visc_face<FT, D, TX, TY, TZ>(P, ring, fx + 1, fy + 1, fz + 1, dxinvT, FF + f, PC::NF);
        }
        __syncthreads();
    }
    // ---- 4. divergence contribution and optional face-flux output
    {
        const int ti = tid % TX, tj = (tid / TX) % TY, tk = tid / (TX * TY);
        const int f = ti + tj * PC::FX + tk * PC::FX * PC::FY;
        const FT dxi = dxinv_of<FT>(B, D);
#pragma unroll
        for (int n = 0; n < 5; ++n) {
            if constexpr (std::is_same<FT, float>::value) {
                // explicit roundings (see sw_split_f32)
                const float df = __fsub_rn(FF[n * PC::NF + f], FF[n * PC::NF + f + PC::FST]);
                acc[n] = (D == 0) ? __fmul_rn(dxi, df) : __fmaf_rn(dxi, df, acc[n]);
            } else {
                FT v = dxi * (FF[n * PC::NF + f] - FF[n * PC::NF + f + PC::FST]);
                acc[n] = (D == 0) ? v : acc[n] + v;
            }
        }
    }
    if (B.has_flux) {
        const View<double>& out = B.flux[D];
        const int fl = B.has_flux;
        const double wdt = (fl & (FLUX_ACC_ALL | FLUX_ACC_PLANES)) ? B.flux_w * (B.dt_ptr ? *B.dt_ptr : B.dt) : 0.0;
        for (int f = tid; f < PC::NF; f += NT) {
            const int fx = f % PC::FX, fy = (f / PC::FX) % PC::FY, fz = f / (PC::FX * PC::FY);
            const int fc[3] = {fx, fy, fz};
            const int gi = i0 + fx, gj = j0 + fy, gk = k0 + fz;
            const int g[3] = {gi, gj, gk};
            bool ok = true;
#pragma unroll
            for (int t = 0; t < 3; ++t) {
                const int lim = B.hi[t] + (t == D ? 1 : 0);
                const int tdim = t == 0 ? TX : (t == 1 ? TY : TZ);
                ok = ok && g[t] <= lim;
                // the tile owns faces 0..T_D-1, plus face T_D at the box's high end
                if (t == D) ok = ok && (fc[t] < tdim || g[t] == B.hi[t] + 1);
            }
            if (ok) {
                if (fl & FLUX_WRITE) {
#pragma unroll
                    for (int n = 0; n < 5; ++n) out(gi, gj, gk, n) = widen<FT>(FF[n * PC::NF + f]);
                } else if (fl & FLUX_ACC_ALL) {
#pragma unroll
                    for (int n = 0; n < 5; ++n)
                        out(gi, gj, gk, n) = __fma_rn(wdt, widen<FT>(FF[n * PC::NF + f]), out(gi, gj, gk, n));
                }
                if ((fl & FLUX_ACC_PLANES) && (g[D] == B.lo[D] || g[D] == B.hi[D] + 1)) {
                    const View<double>& pl = B.fplane[D][g[D] == B.lo[D] ? 0 : 1];
#pragma unroll
                    for (int n = 0; n < 5; ++n)
                        pl(gi, gj, gk, n) = __fma_rn(wdt, widen<FT>(FF[n * PC::NF + f]), pl(gi, gj, gk, n));
                }
            }
        }
    }
    __syncthreads();
}

// One tile (index t over the box list, or over the single box) of the fused
// RHS / stage; the CFL bound of its cells is folded into local_dt.
template <class FT, int TX, int TY, int TZ, bool VISC, bool XS>
__device__ __forceinline__ void rhs_tile(const RegBoxArgs* __restrict__ boxes, const int* __restrict__ tile_start,
                                         int nbox, const RegBoxArgs& single, const DevParm& P, int t,
                                         unsigned char* sbase, uint64_t* bar, uint32_t& phase, bool& abort,
                                         double& local_dt) {
    constexpr int NT = TX * TY * TZ;
    // locate the box of this tile: a single box, or a prefix table over a box list
    int b = 0;
    if (boxes) {
        int lo = 0, hi = nbox - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (tile_start[mid] <= t) lo = mid; else hi = mid - 1;
        }
        b = lo;
        t -= tile_start[b];
    }
    const RegBoxArgs& B = boxes ? boxes[b] : single;
    const int ntx = B.ntile[0], nty = B.ntile[1];
    const int tx = t % ntx, ty = (t / ntx) % nty, tz = t / (ntx * nty);
    const int i0 = B.lo[0] + tx * TX, j0 = B.lo[1] + ty * TY, k0 = B.lo[2] + tz * TZ;

    FT acc[5];
    if constexpr (CrossOn<FT, TX, TY, TZ, VISC, XS>::value) {
        using C = Cross<TX, TY, TZ>;
        double* stage = reinterpret_cast<double*>(sbase);
        float* Q = reinterpret_cast<float*>(sbase + cross_region_a<FT, TX, TY, TZ>());
        const bool staged = B.use_tma != 0;
        if (staged) {
            // region A was last written by the generic proxy (the previous tile's
            // sweeps): order those accesses before this tile's TMA writes
            tma::fence_proxy_async();
            __syncthreads();
            if (threadIdx.x == 0) {
                if (boxes)  // maps of a box table in global memory (a kernel parameter needs no fence)
                    for (int m = 0; m < 4; ++m) tma::fence_tensormap_acquire(&B.tmap[m]);
                const bool stz = !B.zvirt;
                tma::expect_tx(bar, C::BYTES_CXY + (stz ? C::BYTES_Z : 0u));
                const int x = i0 - B.S.b0, y = j0 - B.S.b1, z = k0 - B.S.b2;
                tma::load_4d(stage + C::OC, &B.tmap[0], x, y, z, 0, bar);
                tma::load_4d(stage + C::OXL, &B.tmap[1], x - 4, y, z, 0, bar);
                tma::load_4d(stage + C::OXH, &B.tmap[1], x + TX, y, z, 0, bar);
                tma::load_4d(stage + C::OYL, &B.tmap[2], x, y - 3, z, 0, bar);
                tma::load_4d(stage + C::OYH, &B.tmap[2], x, y + TY, z, 0, bar);
                if (stz) {
                    tma::load_4d(stage + C::OZL, &B.tmap[3], x, y, z - 3, 0, bar);
                    tma::load_4d(stage + C::OZH, &B.tmap[3], x, y, z + TZ, 0, bar);
                }
            }
            const bool done = tc::mbar_wait(bar, phase);
            phase ^= 1u;
            if (!__syncthreads_and(done)) {
                // the bounded wait ran out: report it, give the copies in flight the
                // same time to land, and leave the remaining tiles
                if (threadIdx.x == 0 && P.err) atomicOr(P.err, 2u);
                tc::mbar_wait(bar, phase ^ 1u);
                abort = true;
                return;
            }
        }
        cross_prims<TX, TY, TZ>(B, P, i0, j0, k0, stage, staged, Q);
        __syncthreads();
        FT* F = reinterpret_cast<FT*>(sbase);
        sweep<FT, 0, TX, TY, TZ, VISC, true>(B, P, i0, j0, k0, F, F + 10 * Pencil<0, TX, TY, TZ>::N, nullptr, acc, Q);
        sweep<FT, 1, TX, TY, TZ, VISC, true>(B, P, i0, j0, k0, F, F + 10 * Pencil<1, TX, TY, TZ>::N, nullptr, acc, Q);
        sweep<FT, 2, TX, TY, TZ, VISC, true>(B, P, i0, j0, k0, F, F + 10 * Pencil<2, TX, TY, TZ>::N, nullptr, acc, Q);
    } else if constexpr (CrossPlain<FT, TX, TY, TZ, VISC>::value) {
        FT* F = reinterpret_cast<FT*>(sbase);
        double* Q = F + pencil_elems<TX, TY, TZ>();
        cross_prims_plain<TX, TY, TZ>(B, P, i0, j0, k0, Q);
        __syncthreads();
        sweep<FT, 0, TX, TY, TZ, VISC, true>(B, P, i0, j0, k0, F, F + 10 * Pencil<0, TX, TY, TZ>::N, nullptr, acc, Q);
        sweep<FT, 1, TX, TY, TZ, VISC, true>(B, P, i0, j0, k0, F, F + 10 * Pencil<1, TX, TY, TZ>::N, nullptr, acc, Q);
        sweep<FT, 2, TX, TY, TZ, VISC, true>(B, P, i0, j0, k0, F, F + 10 * Pencil<2, TX, TY, TZ>::N, nullptr, acc, Q);
    } else {
    constexpr int PMAX = pencil_elems<TX, TY, TZ>();
    FT* smem = reinterpret_cast<FT*>(sbase);
    FT* F = smem;
    FT* ring = smem + PMAX;
    if (VISC) {
        using R = Ring<TX, TY, TZ>;
        for (int c = threadIdx.x; c < R::N; c += NT) {
            const int rx = c % R::RX, ry = (c / R::RX) % R::RY, rz = c / (R::RX * R::RY);
            const int gi = i0 + rx - 1, gj = j0 + ry - 1, gk = k0 + rz - 1;
            FT q[7] = {0, 0, 0, 0, 0, 1, 0};
            if (gi <= B.hi[0] + 1 && gj <= B.hi[1] + 1 && gk <= B.hi[2] + 1) {
                int sg;
                Prec<FT>::prims(P, B.S, gi, gj, zmap(B, gk, sg), q);
                if (sg & 1) q[QU] = -q[QU];
                if (sg & 2) q[QV] = -q[QV];
                if (sg & 4) q[QW] = -q[QW];
            }
            ring[c] = q[QU];
            ring[R::N + c] = q[QV];
            ring[2 * R::N + c] = q[QW];
            ring[3 * R::N + c] = q[QT];
        }
        __syncthreads();
    }
    sweep<FT, 0, TX, TY, TZ, VISC>(B, P, i0, j0, k0, F, F + 10 * Pencil<0, TX, TY, TZ>::N, ring, acc);
    sweep<FT, 1, TX, TY, TZ, VISC>(B, P, i0, j0, k0, F, F + 10 * Pencil<1, TX, TY, TZ>::N, ring, acc);
    sweep<FT, 2, TX, TY, TZ, VISC>(B, P, i0, j0, k0, F, F + 10 * Pencil<2, TX, TY, TZ>::N, ring, acc);
    }

    const int ti = threadIdx.x % TX, tj = (threadIdx.x / TX) % TY, tk = threadIdx.x / (TX * TY);
    const int ci = i0 + ti, cj = j0 + tj, ck = k0 + tk;
    const bool valid = ci <= B.hi[0] && cj <= B.hi[1] && ck <= B.hi[2];
    if (valid) {
        double L[5];
#pragma unroll
        for (int n = 0; n < 5; ++n) L[n] = widen<FT>(acc[n]);
        if (P.grav != 0.0) {
            // gravity source after divop, Source/Advance.cpp:331-342
            L[3] = __fma_rn(P.grav, B.S(ci, cj, ck, 0), L[3]);
            L[4] = __fma_rn(P.grav, B.S(ci, cj, ck, 3), L[4]);
        }
        if (B.mode == RHS_WRITE_DSDT) {
#pragma unroll
            for (int n = 0; n < 5; ++n) B.dsdt(ci, cj, ck, n) = L[n];
        } else {
            // fused Shu-Osher stage in FP64: U_out = a U0 + b (U_s + dt L(U_s))
            const double dt = B.dt_ptr ? *B.dt_ptr : B.dt;
            double un[5];
#pragma unroll
            for (int n = 0; n < 5; ++n) {
                double us = B.S(ci, cj, ck, n);
                double u0 = B.U0(ci, cj, ck, n);
                if constexpr (std::is_same<FT, float>::value)  // explicit roundings (see sw_split_f32)
                    un[n] = __fma_rn(B.rk_b, __fma_rn(dt, L[n], us), __dmul_rn(B.rk_a, u0));
                else
                    un[n] = B.rk_a * u0 + B.rk_b * (us + dt * L[n]);
                B.Uout(ci, cj, ck, n) = un[n];
            }
            if (B.cfl_min) {
                const double v = stage_cfl_bound<FT>(P, un, B);
                local_dt = v < local_dt ? v : local_dt;
            }
        }
    }
}

// Tile schedules of one launch over a box list:
//   SCHED_GRID    one CTA per tile (grid = tiles)
//   SCHED_STRIDE  persistent: grid = resident CTAs, CTA c takes tiles c, c + grid, ...
//   SCHED_QUEUE   persistent: CTAs take the next tile from a counter in `queue`
//                 (queue[0] next tile, queue[1] CTAs done); the last CTA to finish
//                 resets both, so every launch starts from zero (graph replays too)
// CTAs per SM that a tile's shared memory admits (228 KB per SM, 1 KB of it
// reserved per CTA; at most 2048 threads), capped at 3: the register budget
// follows from it, so the compiler neither spills below nor plans above the
// occupancy the tile gets (the cap keeps 8^3 FP32 pencil tiles at three CTAs,
// measured faster than two without spills and than four with 32 registers)
template <class FT, int TX, int TY, int TZ, bool VISC, bool XS>
__host__ __device__ constexpr int regular_min_blocks() {
    if (std::is_same<FT, double>::value) return 1;  // the FP64 WENO-Z runs hold a sliding window
    const int b = (int)((228u * 1024u) / (regular_smem_bytes<FT, TX, TY, TZ, VISC, XS>() + 1024u));
    const int t = 2048 / (TX * TY * TZ);
    int m = b < t ? b : t;
    m = m < 3 ? m : 3;
    return m < 1 ? 1 : m;
}

template <class FT, int TX, int TY, int TZ, bool VISC, bool XS>
__global__ void __launch_bounds__(TX* TY* TZ, (regular_min_blocks<FT, TX, TY, TZ, VISC, XS>()))
    k_rhs_regular(const RegBoxArgs* __restrict__ boxes, const int* __restrict__ tile_start,
                  int nbox, const __grid_constant__ RegBoxArgs single, DevParm P, int ntiles, int sched,
                  unsigned* queue) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint64_t tma_bar;
    constexpr bool cross = CrossOn<FT, TX, TY, TZ, VISC, XS>::value;
    // the TMA-staged layout starts at a 128-byte boundary (its size includes the slack)
    unsigned char* sbase =
        cross ? reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127))
              : smem_raw;
    uint32_t phase = 0;
    bool abort = false;
    if constexpr (cross) {
        if (threadIdx.x == 0) tc::mbar_init(&tma_bar, 1);
        __syncthreads();
    }
    double local_dt = __longlong_as_double(0x7FF0000000000000LL);
    unsigned long long* cfl = boxes ? boxes[0].cfl_min : single.cfl_min;  // one target per stage
    if (sched == SCHED_GRID) {
        rhs_tile<FT, TX, TY, TZ, VISC, XS>(boxes, tile_start, nbox, single, P, blockIdx.x, sbase, &tma_bar, phase, abort,
                                       local_dt);
    } else if (sched == SCHED_STRIDE) {
        for (int t = blockIdx.x; t < ntiles && !abort; t += gridDim.x) {
            rhs_tile<FT, TX, TY, TZ, VISC, XS>(boxes, tile_start, nbox, single, P, t, sbase, &tma_bar, phase, abort,
                                           local_dt);
            __syncthreads();
        }
    } else {
        __shared__ int next;
        for (;;) {
            if (threadIdx.x == 0) next = (int)atomicAdd(&queue[0], 1u);
            __syncthreads();
            const int t = next;
            __syncthreads();
            if (t >= ntiles || abort) break;
            rhs_tile<FT, TX, TY, TZ, VISC, XS>(boxes, tile_start, nbox, single, P, t, sbase, &tma_bar, phase, abort,
                                           local_dt);
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            __threadfence();
            if (atomicAdd(&queue[1], 1u) == gridDim.x - 1) {
                queue[0] = 0u;
                queue[1] = 0u;
                __threadfence();
            }
        }
    }
    if (cfl) block_min_atomic(local_dt, cfl);
}

template <class FT, int TX, int TY, int TZ, bool VISC, bool XS>
static ocfd_status launch_t(const RegBoxArgs* d_boxes, const int* d_tile_start, int nbox,
                            const RegBoxArgs& single, int ntiles, const DevParm& P,
                            cudaStream_t st, int sched, unsigned* queue) {
    constexpr int NT = TX * TY * TZ;
    constexpr size_t smem = regular_smem_bytes<FT, TX, TY, TZ, VISC, XS>();
    auto kern = k_rhs_regular<FT, TX, TY, TZ, VISC, XS>;
    if (smem > kMaxSmem) return fail(OCFD_BAD_ARG, "regular RHS tile does not fit shared memory in this mode");
    if (ntiles <= 0) return OCFD_OK;
    if (sched == SCHED_QUEUE && !queue) return fail(OCFD_BAD_ARG, "regular RHS: work-queue schedule without a queue");
    int grid = ntiles;
    if (sched != SCHED_GRID) {
        // resident CTAs of this shape over the whole GPU (cached per instantiation)
        static int resident = 0;
        if (resident == 0) {
            int per_sm = 0, dev = 0, sms = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem) != cudaSuccess) per_sm = 1;
            resident = std::max(1, per_sm) * std::max(1, sms);
        }
        grid = std::min(ntiles, resident);
    }
    kern<<<grid, NT, smem, st>>>(d_boxes, d_tile_start, nbox, single, P, ntiles, sched, queue);
    return check_launch("k_rhs_regular");
}

template <class FT, int TX, int TY, int TZ, bool VISC, bool XS>
static bool configure_one() {
    const size_t smem = regular_smem_bytes<FT, TX, TY, TZ, VISC, XS>();
    if (smem > kMaxSmem) return true;  // shape not offered in this mode
    return cudaFuncSetAttribute(k_rhs_regular<FT, TX, TY, TZ, VISC, XS>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess;
}

// Every compiled tile: index (position in kRegularTiles), shape, and whether it
// is the TMA-staged variant (XS) of its shape.  A staged index runs the staged
// kernel only in the inviscid FP32-flux form; in every other mode it runs the
// pencil kernel of its shape (the same instantiation as the plain index).
#define OCFD_REGULAR_TILES(X)                                                                              \
    X(0, 8, 8, 8, false) X(1, 8, 8, 4, false) X(2, 16, 8, 4, false) X(3, 16, 16, 2, false) X(4, 32, 8, 2, false) \
        X(5, 16, 8, 2, false) X(6, 8, 8, 8, true) X(7, 8, 8, 4, true) X(8, 16, 8, 4, true)

template <class FT>
struct StagedIn {  // the staged variants exist in the FP32-flux form only
    static constexpr bool value = std::is_same<FT, float>::value;
};

template <class FT>
static ocfd_status configure_all() {
    bool ok = true;
#define OCFD_CONF(I, X, Y, Z, XS) \
    ok = ok && configure_one<FT, X, Y, Z, false, XS && StagedIn<FT>::value>() && configure_one<FT, X, Y, Z, true, false>();
    OCFD_REGULAR_TILES(OCFD_CONF)
#undef OCFD_CONF
    if (!ok) return check_launch("configure regular RHS kernels");
    return OCFD_OK;
}

template <class FT>
static bool tile_fits(int tile, bool visc) {
    size_t b = 0;
    switch (tile) {
#define OCFD_FIT(I, X, Y, Z, XS)                                                                                \
    case I:                                                                                                     \
        b = visc ? regular_smem_bytes<FT, X, Y, Z, true, false>()                                               \
                 : regular_smem_bytes<FT, X, Y, Z, false, XS && StagedIn<FT>::value>();                         \
        break;
        OCFD_REGULAR_TILES(OCFD_FIT)
#undef OCFD_FIT
        default:
            return false;
    }
    return b <= kMaxSmem;
}

template <class FT>
static ocfd_status launch_any(int tile, bool visc, const RegBoxArgs* d_boxes, const int* d_tile_start,
                              int nbox, const RegBoxArgs& single, int ntiles, const DevParm& P,
                              cudaStream_t st, int sched = SCHED_GRID, unsigned* queue = nullptr) {
    switch (tile) {
#define OCFD_CASE(I, X, Y, Z, XS)                                                                               \
    case I:                                                                                                     \
        return visc ? launch_t<FT, X, Y, Z, true, false>(d_boxes, d_tile_start, nbox, single, ntiles, P, st,    \
                                                         sched, queue)                                          \
                    : launch_t<FT, X, Y, Z, false, XS && StagedIn<FT>::value>(d_boxes, d_tile_start, nbox,      \
                                                                              single, ntiles, P, st, sched, queue);
        OCFD_REGULAR_TILES(OCFD_CASE)
#undef OCFD_CASE
    }
    return fail(OCFD_BAD_ARG, "regular RHS: bad tile index");
}

}  // namespace ocfd
