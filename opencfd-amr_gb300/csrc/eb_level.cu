// Embedded boundary over a level of boxes (ideal gas).
//
// The box loop of EBR::compute_dSdt (Source/Advance.cpp:201-342) picks a scheme
// per box: all cells covered -> dSdt = 0 (:213-214); grow(bx, NUM_GROW) free of
// cut and covered cells -> the regular WENO-Z chain (:231); otherwise the
// cut-cell scheme eb_compute_dSdt_box (Source/EB/AdvanceBox.cpp:16-228).  Here
// the regular boxes stay in the fused tile kernel, and all cut and covered boxes
// of the level run as one launch per RK stage of k_ebl_tile: one CTA per 8x8x4
// tile, primitives (c2prim) over grow(tile, 2), or over the tile's cross in
// inviscid stages, the tile's faces in x, y and z
// (MUSCL-minmod states, Van Leer flux, EB viscous flux; RK-weighted
// area-fraction fluxes into the flux registers of an AMR level) in shared
// memory, then per cell the cut-cell divergence with the wall flux, negated
// (zero in covered boxes), fused with the Shu-Osher stage update and the CFL
// bound of the new state.  In the mixed form (OCFD_FLUX_FP32, inviscid) the
// primitives (from the narrowed state), the face states, the Van Leer flux, the
// cut-cell divergence with the slip-wall pressure flux and the CFL bound are
// FP32; the RK stage update stays FP64.  Tiles are addressed through a prefix
// table over the boxes.
//
// Geometry.  AMReX EB2 (Source/Geometry.cpp:9-29) is absent.  For a body
// extruded along z the cut-cell data do not depend on z, so each box keeps 2D
// arrays over grow(bx, 5) in x and y, read through views with kstride 0:
//   vfrac  volume fraction: fraction of nsub x nsub sub-cell centres in the fluid
//   apx    x-face area fraction: fraction of nsub points along the face
//   apy    y-face area fraction
//   apz    z faces: the column's volume fraction
//   flag   EBCellFlag word: bits 0-1 type (0 regular, 1 cut, 3 covered), bits
//          4 + (i+1) + 3(j+1) + 9(k+1) connectivity to neighbour (i, j, k): a
//          cut cell is connected to a neighbour that is not covered, through an
//          open face (area fraction > 0) for face neighbours; regular cells
//          carry all 27 bits; neighbours outside the stored region count as
//          covered.  A cell is regular when its volume fraction and the area
//          fractions of its six faces are 1.
// The sample points, their arithmetic (IEEE round-to-nearest, no contraction)
// and the reductions are those of the fixture generator the tests compare with,
// so the geometry is identical to it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <tuple>
#include <type_traits>
#include <vector>

#include "eb_level.h"
#include "eb_physics.cuh"
#include "weno_f32.cuh"

namespace ocfd {

constexpr int EB_GG = EB_GEOM_GROW;

struct GeoTag {
    int lo[2];         // first cell (x, y) of the stored region, grow(bx, 5)
    int gx, gy;        // stored cells
    long long off_vf, off_ax, off_ay, off_fl;
};

struct EbShape {
    int kind, nsub;
    double cx, cy, r;
    double plo[2], dx[2];
};

__device__ __forceinline__ double phi_of(const EbShape& s, double x, double y) {
    const double a = __dsub_rn(x, s.cx), b = __dsub_rn(y, s.cy);
    return __dsub_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(s.r, s.r));
}
// sample coordinate prob_lo + (i + (m + 1/2) / nsub) dx, and the face coordinate prob_lo + i dx
__device__ __forceinline__ double sample_at(const EbShape& s, int d, int i, int m) {
    const double sm = __ddiv_rn(__dadd_rn((double)m, 0.5), (double)s.nsub);
    return __dadd_rn(s.plo[d], __dmul_rn(__dadd_rn((double)i, sm), s.dx[d]));
}
__device__ __forceinline__ double face_at(const EbShape& s, int d, int i) {
    return __dadd_rn(s.plo[d], __dmul_rn((double)i, s.dx[d]));
}

// volume and area fractions of every stored cell / face
__global__ void k_geom_frac(const GeoTag* __restrict__ tags, const long long* __restrict__ start, int ntag,
                            long long total, EbShape sh, double* geo) {
    const int ns = sh.nsub;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int t = find_tag<GeoTag>(start, ntag, idx);
        const GeoTag& T = tags[t];
        const long long loc = idx - start[t];
        const int W = T.gx + 1;
        const int li = (int)(loc % W), lj = (int)(loc / W);
        const int i = T.lo[0] + li, j = T.lo[1] + lj;
        if (li < T.gx && lj < T.gy) {
            int cnt = 0;
            for (int b = 0; b < ns; ++b) {
                const double y = sample_at(sh, 1, j, b);
                for (int a = 0; a < ns; ++a) cnt += phi_of(sh, sample_at(sh, 0, i, a), y) > 0.0;
            }
            geo[T.off_vf + li + (long long)lj * T.gx] = __ddiv_rn((double)cnt, (double)(ns * ns));
        }
        if (lj < T.gy) {
            const double xf = face_at(sh, 0, i);
            int cnt = 0;
            for (int b = 0; b < ns; ++b) cnt += phi_of(sh, xf, sample_at(sh, 1, j, b)) > 0.0;
            geo[T.off_ax + li + (long long)lj * (T.gx + 1)] = __ddiv_rn((double)cnt, (double)ns);
        }
        if (li < T.gx) {
            const double yf = face_at(sh, 1, j);
            int cnt = 0;
            for (int a = 0; a < ns; ++a) cnt += phi_of(sh, sample_at(sh, 0, i, a), yf) > 0.0;
            geo[T.off_ay + li + (long long)lj * T.gx] = __ddiv_rn((double)cnt, (double)ns);
        }
    }
}

__host__ __device__ constexpr int conn_bit(int i, int j, int k) { return 4 + (i + 1) + 3 * (j + 1) + 9 * (k + 1); }

// flag words of every stored cell; per box the count of cells that are not
// regular inside grow(bx, 4) and of covered cells inside bx (class test)
__global__ void k_geom_flag(const GeoTag* __restrict__ tags, const long long* __restrict__ start, int ntag,
                            long long total, const double* __restrict__ geo, uint32_t* flag,
                            unsigned long long* counts) {
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int t = find_tag<GeoTag>(start, ntag, idx);
        const GeoTag& T = tags[t];
        const long long loc = idx - start[t];
        const int li = (int)(loc % T.gx), lj = (int)(loc / T.gx);
        const double* vf = geo + T.off_vf;
        const double* ax = geo + T.off_ax;
        const double* ay = geo + T.off_ay;
        auto VF = [&](int a, int b) { return vf[a + (long long)b * T.gx]; };
        auto AX = [&](int a, int b) { return ax[a + (long long)b * (T.gx + 1)]; };
        auto AY = [&](int a, int b) { return ay[a + (long long)b * T.gx]; };
        const double v = VF(li, lj);
        const bool covered = v <= 0.0;
        const bool full = v >= 1.0;
        const bool open = AX(li, lj) >= 1.0 && AX(li + 1, lj) >= 1.0 && AY(li, lj) >= 1.0 && AY(li, lj + 1) >= 1.0;
        uint32_t w;
        if (full && open) {
            w = 0u;
            for (int b = 0; b < 27; ++b) w |= 1u << (4 + b);
        } else if (covered) {
            w = 3u;
        } else {
            w = 1u;
            for (int dk = -1; dk <= 1; ++dk)
                for (int dj = -1; dj <= 1; ++dj)
                    for (int di = -1; di <= 1; ++di) {
                        const int ni = li + di, nj = lj + dj;
                        const bool inside = ni >= 0 && ni < T.gx && nj >= 0 && nj < T.gy;
                        bool ok = inside && !(VF(ni, nj) <= 0.0);
                        const int nface = (di != 0) + (dj != 0) + (dk != 0);
                        if (ok && nface == 1) {
                            double a;
                            if (di) a = di > 0 ? AX(li + 1, lj) : AX(li, lj);
                            else if (dj) a = dj > 0 ? AY(li, lj + 1) : AY(li, lj);
                            else a = v;
                            ok = a > 0.0;
                        }
                        if (ok) w |= 1u << conn_bit(di, dj, dk);
                    }
        }
        flag[T.off_fl + loc] = w;
        // class counts: grow(bx, 4) is the stored region less its outer ring
        if (li >= 1 && li < T.gx - 1 && lj >= 1 && lj < T.gy - 1 && (w & 3u) != 0u)
            atomicAdd(&counts[2 * t], 1ull);
        if (li >= EB_GG && li < T.gx - EB_GG && lj >= EB_GG && lj < T.gy - EB_GG && covered)
            atomicAdd(&counts[2 * t + 1], 1ull);
    }
}

// ------------------------------------------------------------------ stages
struct EbStageBox {
    View<const double> S, U0;
    View<double> Uout;
    View<const uint32_t> flag;
    View<const double> vfrac, ap[3];
    int lo[3], hi[3];
    double rk_a, rk_b;
    int covered;
    int has_flux;  // FLUX_ACC_ALL / FLUX_ACC_PLANES
    double flux_w;
    View<double> creg[3];
    View<double> fplane[3][2];
};

struct EbStageArgs {
    const EbStageBox* boxes;
    int nbox;
    double dxinv[3], dx[3];
    float dxinv_f[3], dx_f[3];  // FP32 copies for the mixed form
    const double* dt_ptr;
    unsigned long long* cfl_min;
    int visc, redist;
};

// ------------------------------------------------------------ fused tile kernel
// The batched cut-cell stage as one kernel: one CTA per 8x8x4 tile of a cut or
// covered box.  The primitives (over grow(tile, 2), or over the tile's cross in
// an inviscid stage) and the tile's face fluxes in x, y and z stay in shared
// memory; each cell thread then forms the cut-cell divergence with the wall flux
// (Source/EB/EBkernels.H:216-338, negated, the small-cell rescale of flux_redist
// :341-377), the Shu-Osher stage and the CFL bound.  Only the state (read once
// per cell of that region), the stage input U0, the output and the z-invariant
// geometry touch memory: no primitive or face-flux scratch round trip.  A face
// on a tile boundary is computed by both tiles and added to the flux registers
// by the one that owns it (faces 0 .. T_D - 1 of the tile, plus the box's high
// face), so that every face is accumulated once.  The per-box form
// (OCFD_PER_BOX) launches the same kernel box by box.
constexpr int EBT_X = 8, EBT_Y = 8, EBT_Z = 4, EBT_N = EBT_X * EBT_Y * EBT_Z;
constexpr int EBQ_X = EBT_X + 4, EBQ_Y = EBT_Y + 4, EBQ_Z = EBT_Z + 4, EBQ_N = EBQ_X * EBQ_Y * EBQ_Z;
constexpr int EBF_N0 = (EBT_X + 1) * EBT_Y * EBT_Z, EBF_N1 = EBT_X * (EBT_Y + 1) * EBT_Z,
              EBF_N2 = EBT_X * EBT_Y * (EBT_Z + 1);

// Inviscid stages keep only the cross of the tile - the tile and 2 cells on
// each side along x, y and z, the cells the faces' MUSCL stencils read - and 6
// primitive planes (the Van Leer flux reads no temperature): 768 cells against
// 1152 of grow(tile, 2).  The viscous stage (FP64) keeps grow(tile, 2) whole
// and 7 planes (its face stress reads transverse neighbours).
constexpr int EBX_NC = EBT_X * EBT_Y * EBT_Z, EBX_NX = 4 * EBT_Y * EBT_Z, EBX_NY = 4 * EBT_X * EBT_Z,
              EBX_NZ = 4 * EBT_X * EBT_Y, EBX_N = EBX_NC + EBX_NX + EBX_NY + EBX_NZ;

template <bool F32>
__host__ __device__ constexpr size_t ebt_smem_bytes(bool visc = true) {
    return (F32 ? sizeof(float) : sizeof(double)) *
           ((visc ? 7 * EBQ_N : 6 * EBX_N) + 5 * (EBF_N0 + EBF_N1 + EBF_N2));
}

// primitive plane of component m (cross layout: no temperature plane)
__device__ __forceinline__ int ebt_plane(bool cross, int m) { return cross && m > QT ? m - 1 : m; }

// shared-memory index of tile-local cell (x, y, z), -2 <= x < EBT_X + 2 etc.;
// in the cross layout at most one coordinate lies outside the tile
__device__ __forceinline__ int ebt_q(bool cross, int x, int y, int z) {
    if (!cross) return (x + 2) + (y + 2) * EBQ_X + (z + 2) * EBQ_X * EBQ_Y;
    if (x < 0 || x >= EBT_X) return EBX_NC + (x < 0 ? x + 2 : x - EBT_X + 2) + 4 * (y + EBT_Y * z);
    if (y < 0 || y >= EBT_Y) return EBX_NC + EBX_NX + x + EBT_X * ((y < 0 ? y + 2 : y - EBT_Y + 2) + 4 * z);
    if (z < 0 || z >= EBT_Z) return EBX_NC + EBX_NX + EBX_NY + x + EBT_X * (y + EBT_Y * (z < 0 ? z + 2 : z - EBT_Z + 2));
    return x + EBT_X * (y + EBT_Y * z);
}

// tile-local cell of index c of the cross layout (the inverse of ebt_q)
__device__ __forceinline__ void ebt_cross_cell(int c, int& x, int& y, int& z) {
    if (c < EBX_NC) {
        x = c % EBT_X;
        y = (c / EBT_X) % EBT_Y;
        z = c / (EBT_X * EBT_Y);
    } else if (c < EBX_NC + EBX_NX) {
        const int r = c - EBX_NC, h = r % 4;
        y = (r / 4) % EBT_Y;
        z = r / (4 * EBT_Y);
        x = h < 2 ? h - 2 : EBT_X + h - 2;
    } else if (c < EBX_NC + EBX_NX + EBX_NY) {
        const int r = c - EBX_NC - EBX_NX, h = (r / EBT_X) % 4;
        x = r % EBT_X;
        z = r / (4 * EBT_X);
        y = h < 2 ? h - 2 : EBT_Y + h - 2;
    } else {
        const int r = c - EBX_NC - EBX_NX - EBX_NY, h = r / (EBT_X * EBT_Y);
        x = r % EBT_X;
        y = (r / EBT_X) % EBT_Y;
        z = h < 2 ? h - 2 : EBT_Z + h - 2;
    }
}

// faces of direction D of the tile at (i0, j0, k0) of box B into sf (5 x EBF_N[D])
template <bool F32, int D>
__device__ __forceinline__ void ebt_faces(const EbStageArgs& A, const EbStageBox& B, const DevParm& P, int i0,
                                          int j0, int k0, double dt,
                                          typename std::conditional<F32, float, double>::type* sq,
                                          typename std::conditional<F32, float, double>::type* sf) {
    using FT = typename std::conditional<F32, float, double>::type;
    constexpr int FX = EBT_X + (D == 0), FY = EBT_Y + (D == 1), FZ = EBT_Z + (D == 2), NF = FX * FY * FZ;
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const bool cross = !A.visc;
    const int NP = cross ? EBX_N : EBQ_N;
    for (int f = threadIdx.x; f < NF; f += EBT_N) {
        const int fx = f % FX, fy = (f / FX) % FY, fz = f / (FX * FY);
        const int i = i0 + fx, j = j0 + fy, k = k0 + fz;
        if (i > B.hi[0] + di || j > B.hi[1] + dj || k > B.hi[2] + dk) continue;
        const uint32_t fl = B.flag(i, j, k);
        // the face's four stencil cells along D (offsets -2, -1, 0, +1)
        const int s0 = ebt_q(cross, fx - 2 * di, fy - 2 * dj, fz - 2 * dk);
        const int s1 = ebt_q(cross, fx - di, fy - dj, fz - dk);
        const int s2 = ebt_q(cross, fx, fy, fz);
        const int s3 = ebt_q(cross, fx + di, fy + dj, fz + dk);
        double flx[5];
        if (F32) {
            const bool cm1 = eb_conn(fl, -di, -dj, -dk), cm2 = eb_conn(fl, -2 * di, -2 * dj, -2 * dk),
                       cp1 = eb_conn(fl, di, dj, dk);
            float ql[7], qr[7], ff[5];
#pragma unroll
            for (int m = 0; m < 7; ++m) {
                if (m == QT) {
                    ql[m] = qr[m] = 0.0f;
                    continue;
                }
                const FT* pm = sq + ebt_plane(cross, m) * NP;
                const float vm2 = pm[s0], vm1 = pm[s1], v0 = pm[s2], vp1 = pm[s3];
                float l = vm1, r = v0;
                if (cm1) {
                    if (cm2) l = vm1 + 0.5f * minmod<float>(v0 - vm1, vm1 - vm2);
                    if (cp1) r = v0 - 0.5f * minmod<float>(vp1 - v0, v0 - vm1);
                }
                ql[m] = l;
                qr[m] = r;
            }
            vanleer_g<float>(P.f_smallp, P.f_gamma, P.f_vl_rg, P.f_vl_rg21, P.f_vl_ggm1, ql, qr, D, ff);
#pragma unroll
            for (int m = 0; m < 5; ++m) {
                sf[m * NF + f] = ff[m];
                flx[m] = f2d_bits(ff[m]);
            }
        } else {
            double ql[7], qr[7];
#pragma unroll
            for (int m = 0; m < 7; ++m) {
                if (m == QT) {  // the Van Leer flux does not read the temperature
                    ql[m] = qr[m] = 0.0;
                    continue;
                }
                const FT* pm = sq + ebt_plane(cross, m) * NP;
                eb_recon(fl, D, (double)pm[s0], (double)pm[s1], (double)pm[s2], (double)pm[s3], ql[m], qr[m]);
            }
            vanleer_g<double>(P.smallp, P.gamma, P.vl_rg, P.vl_rg21, P.vl_ggm1, ql, qr, D, flx);
            if (A.visc) {
                const View<const double> qv{reinterpret_cast<const double*>(sq), EBQ_X, (long long)EBQ_X * EBQ_Y,
                                            EBQ_N, i0 - 2, j0 - 2, k0 - 2};
                eb_visc_face(P, qv, B.flag, D, i, j, k, A.dxinv, flx, 1, false, 0, 0, 0);
            }
#pragma unroll
            for (int m = 0; m < 5; ++m) sf[m * NF + f] = flx[m];
        }
        if (B.has_flux) {
            const int g = D == 0 ? i : (D == 1 ? j : k);
            const int fd = D == 0 ? fx : (D == 1 ? fy : fz);
            constexpr int TD = D == 0 ? EBT_X : (D == 1 ? EBT_Y : EBT_Z);
            if (fd < TD || g == B.hi[D] + 1) {
                const double w = B.flux_w * dt * B.ap[D](i, j, k);
                if (B.has_flux & FLUX_ACC_ALL) {
#pragma unroll
                    for (int m = 0; m < 5; ++m) B.creg[D](i, j, k, m) += w * flx[m];
                }
                if ((B.has_flux & FLUX_ACC_PLANES) && (g == B.lo[D] || g == B.hi[D] + 1)) {
                    const View<double>& pl = B.fplane[D][g == B.lo[D] ? 0 : 1];
#pragma unroll
                    for (int m = 0; m < 5; ++m) pl(i, j, k, m) += w * flx[m];
                }
            }
        }
    }
}

template <bool F32>
__global__ void __launch_bounds__(EBT_N) k_ebl_tile(EbStageArgs A, const int* __restrict__ tstart, DevParm P) {
    using FT = typename std::conditional<F32, float, double>::type;
    extern __shared__ __align__(16) unsigned char ebt_raw[];
    FT* sq = reinterpret_cast<FT*>(ebt_raw);
    const bool cross = !A.visc;
    const int NP = cross ? EBX_N : EBQ_N;
    FT* sf0 = sq + (cross ? 6 * EBX_N : 7 * EBQ_N);
    FT* sf1 = sf0 + 5 * EBF_N0;
    FT* sf2 = sf1 + 5 * EBF_N1;
    const double dt = *A.dt_ptr;
    double local_dt = __longlong_as_double(0x7FF0000000000000LL);
    // the box of this tile (prefix table over the cut / covered boxes)
    int t = blockIdx.x;
    int lo = 0, hi = A.nbox - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tstart[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const EbStageBox& B = A.boxes[lo];
    t -= tstart[lo];
    const int ntx = (B.hi[0] - B.lo[0] + EBT_X) / EBT_X, nty = (B.hi[1] - B.lo[1] + EBT_Y) / EBT_Y;
    const int i0 = B.lo[0] + (t % ntx) * EBT_X, j0 = B.lo[1] + ((t / ntx) % nty) * EBT_Y,
              k0 = B.lo[2] + (t / (ntx * nty)) * EBT_Z;
    const int tid = threadIdx.x;
    if (!B.covered) {
        // 1. primitives over the tile's cross (inviscid) or grow(tile, 2)
        // (viscous), within the box's grow(bx, 2)
        for (int c = tid; c < NP; c += EBT_N) {
            int qx, qy, qz;
            if (cross) {
                ebt_cross_cell(c, qx, qy, qz);
            } else {
                qx = c % EBQ_X - 2;
                qy = (c / EBQ_X) % EBQ_Y - 2;
                qz = c / (EBQ_X * EBQ_Y) - 2;
            }
            const int i = i0 + qx, j = j0 + qy, k = k0 + qz;
            if (i > B.hi[0] + 2 || j > B.hi[1] + 2 || k > B.hi[2] + 2) continue;
            if (F32) {
                const float g = P.f_gamma;
                const float u0 = d2f_bits(B.S(i, j, k, 0)), u1 = d2f_bits(B.S(i, j, k, 1)),
                            u2 = d2f_bits(B.S(i, j, k, 2)), u3 = d2f_bits(B.S(i, j, k, 3)),
                            u4 = d2f_bits(B.S(i, j, k, 4));
                const float rho = fmaxf(u0, P.f_smallr);
                const float rhoinv = __frcp_rn(rho);
                const float ux = u1 * rhoinv, uy = u2 * rhoinv, uz = u3 * rhoinv;
                const float p = fmaxf((g - 1.0f) * (u4 - rho * (0.5f * (ux * ux + uy * uy + uz * uz))), P.f_smallp);
                sq[QRHO * NP + c] = rho;
                sq[QU * NP + c] = ux;
                sq[QV * NP + c] = uy;
                sq[QW * NP + c] = uz;
                sq[QPRES * NP + c] = p;
                sq[ebt_plane(cross, QC) * NP + c] = sqrtf(g * p * rhoinv);
            } else {
                double q[7];
                c2prim_ideal_fast(P, B.S(i, j, k, 0), B.S(i, j, k, 1), B.S(i, j, k, 2), B.S(i, j, k, 3),
                                  B.S(i, j, k, 4), q);
#pragma unroll
                for (int m = 0; m < 7; ++m)
                    if (!(cross && m == QT)) sq[ebt_plane(cross, m) * NP + c] = q[m];
            }
        }
        __syncthreads();
        // 2. face fluxes of the tile in x, y, z
        ebt_faces<F32, 0>(A, B, P, i0, j0, k0, dt, sq, sf0);
        ebt_faces<F32, 1>(A, B, P, i0, j0, k0, dt, sq, sf1);
        ebt_faces<F32, 2>(A, B, P, i0, j0, k0, dt, sq, sf2);
        __syncthreads();
    }
    // 3. cut-cell divergence, stage and CFL bound per cell
    const int ti = tid % EBT_X, tj = (tid / EBT_X) % EBT_Y, tk = tid / (EBT_X * EBT_Y);
    const int i = i0 + ti, j = j0 + tj, k = k0 + tk;
    if (i <= B.hi[0] && j <= B.hi[1] && k <= B.hi[2]) {
        // face fluxes of the cell: low and high face per direction, component stride
        const int fxl = ti + tj * (EBT_X + 1) + tk * (EBT_X + 1) * EBT_Y;
        const int fyl = ti + tj * EBT_X + tk * EBT_X * (EBT_Y + 1);
        const int fzl = ti + tj * EBT_X + tk * EBT_X * EBT_Y;
        const int qc = ebt_q(cross, ti, tj, tk);  // the cell in the primitive planes
        auto FXm = [&](int m) { return sf0[m * EBF_N0 + fxl]; };
        auto FXp = [&](int m) { return sf0[m * EBF_N0 + fxl + 1]; };
        auto FYm = [&](int m) { return sf1[m * EBF_N1 + fyl]; };
        auto FYp = [&](int m) { return sf1[m * EBF_N1 + fyl + EBT_X]; };
        auto FZm = [&](int m) { return sf2[m * EBF_N2 + fzl]; };
        auto FZp = [&](int m) { return sf2[m * EBF_N2 + fzl + EBT_X * EBT_Y]; };
        double L[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        if (!B.covered) {
            const uint32_t f = B.flag(i, j, k);
            if (F32) {
                float out[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
                const float vf = d2f_bits(B.vfrac(i, j, k));
                if (eb_regular(f)) {
#pragma unroll
                    for (int m = 0; m < 5; ++m)
                        out[m] = A.dxinv_f[0] * ((float)FXp(m) - (float)FXm(m)) +
                                 A.dxinv_f[1] * ((float)FYp(m) - (float)FYm(m)) +
                                 A.dxinv_f[2] * ((float)FZp(m) - (float)FZm(m));
                } else if (!eb_covered(f)) {
                    const float tmp = __fdividef(A.dxinv_f[0], vf);
                    const float axm = d2f_bits(B.ap[0](i, j, k)), axp = d2f_bits(B.ap[0](i + 1, j, k));
                    const float aym = d2f_bits(B.ap[1](i, j, k)), ayp = d2f_bits(B.ap[1](i, j + 1, k));
                    const float azm = d2f_bits(B.ap[2](i, j, k)), azp = d2f_bits(B.ap[2](i, j, k + 1));
#pragma unroll
                    for (int m = 0; m < 5; ++m)
                        out[m] = tmp * (axp * (float)FXp(m) - axm * (float)FXm(m) + ayp * (float)FYp(m) -
                                        aym * (float)FYm(m) + azp * (float)FZp(m) - azm * (float)FZm(m));
                    const float pr = (float)sq[QPRES * NP + qc];
                    out[1] += (axm - axp) * pr * tmp;
                    out[2] += (aym - ayp) * pr * tmp;
                    out[3] += (azm - azp) * pr * tmp;
                }
                const bool rescale = A.redist && vf < 0.5f && vf > 0.0f;
#pragma unroll
                for (int m = 0; m < 5; ++m) L[m] = f2d_bits(rescale ? -(vf * out[m]) : -out[m]);
            } else {
                const double vf = B.vfrac(i, j, k);
                double out[5];
                if (eb_covered(f)) {
#pragma unroll
                    for (int m = 0; m < 5; ++m) out[m] = 0.0;
                } else if (eb_regular(f)) {
#pragma unroll
                    for (int m = 0; m < 5; ++m)
                        out[m] = A.dxinv[0] * ((double)FXp(m) - (double)FXm(m)) +
                                 A.dxinv[1] * ((double)FYp(m) - (double)FYm(m)) +
                                 A.dxinv[2] * ((double)FZp(m) - (double)FZm(m));
                } else {
                    const double tmp = A.dxinv[0] / vf;
                    const double axm = B.ap[0](i, j, k), axp = B.ap[0](i + 1, j, k);
                    const double aym = B.ap[1](i, j, k), ayp = B.ap[1](i, j + 1, k);
                    const double azm = B.ap[2](i, j, k), azp = B.ap[2](i, j, k + 1);
#pragma unroll
                    for (int m = 0; m < 5; ++m)
                        out[m] = tmp * (axp * (double)FXp(m) - axm * (double)FXm(m) + ayp * (double)FYp(m) -
                                        aym * (double)FYm(m) + azp * (double)FZp(m) - azm * (double)FZm(m));
                    double fw[5];
                    const double pr = (double)sq[QPRES * NP + qc];
                    if (!A.visc) {
                        // slip-wall pressure flux, EBkernels.H:305-311
                        fw[0] = 0.0;
                        fw[1] = (axm - axp) * pr;
                        fw[2] = (aym - ayp) * pr;
                        fw[3] = (azm - azp) * pr;
                        fw[4] = 0.0;
                    } else {
                        // eb_wallflux, EBkernels.H:173-214
                        const double d = (double)sq[QRHO * NP + qc], u = (double)sq[QU * NP + qc],
                                     v = (double)sq[QV * NP + qc], w = (double)sq[QW * NP + qc],
                                     cs = (double)sq[QC * NP + qc];
                        const double apnorm = sqrt((axm - axp) * (axm - axp) + (aym - ayp) * (aym - ayp) +
                                                   (azm - azp) * (azm - azp));
                        const double un = u * (axm - axp) + v * (aym - ayp) + w * (azm - azp);
                        const double lambda0 = fabs(un) + cs * apnorm;
                        const double gamma = P.gamma;
                        const double E0 = pr / (gamma - 1) + 0.50 * d * (u * u + v * v + w * w);
                        double fpw[5], fmw[5];
                        fpw[0] = 0.5 * (d * un + lambda0 * d);
                        fpw[1] = 0.5 * (d * u * un + (axm - axp) * pr + lambda0 * d * u);
                        fpw[2] = 0.5 * (d * v * un + (aym - ayp) * pr + lambda0 * d * v);
                        fpw[3] = 0.5 * (d * w * un + (azm - azp) * pr + lambda0 * d * w);
                        fpw[4] = 0.5 * ((E0 + pr) * un + lambda0 * E0);
                        fmw[0] = 0.5 * (d * (-un) - lambda0 * d);
                        fmw[1] = fpw[1];
                        fmw[2] = fpw[2];
                        fmw[3] = fpw[3];
                        fmw[4] = 0.5 * (-(E0 + pr) * un - lambda0 * E0);
#pragma unroll
                        for (int m = 0; m < 5; ++m) fw[m] = fpw[m] + fmw[m];
                    }
#pragma unroll
                    for (int m = 0; m < 5; ++m) out[m] += fw[m] * tmp;
                }
                const bool rescale = A.redist && vf < 0.5 && vf > 0.0;
#pragma unroll
                for (int m = 0; m < 5; ++m) {
                    const double divc = out[m] * -1.0;
                    L[m] = rescale ? vf * divc : divc;
                }
            }
        }
        double un[5];
#pragma unroll
        for (int n = 0; n < 5; ++n) {
            const double us = B.S(i, j, k, n);
            const double u0 = B.U0(i, j, k, n);
            un[n] = B.rk_a * u0 + B.rk_b * (us + dt * L[n]);
            B.Uout(i, j, k, n) = un[n];
        }
        if (A.cfl_min) {
            double v;
            if (F32) {
                const float g = P.f_gamma;
                const float rho = d2f_bits(un[0]);
                const float rhoinv = __frcp_rn(fmaxf(rho, P.f_smallr));
                const float vx = d2f_bits(un[1]) * rhoinv, vy = d2f_bits(un[2]) * rhoinv, vz = d2f_bits(un[3]) * rhoinv;
                const float p = fmaxf((g - 1.0f) * (d2f_bits(un[4]) - 0.5f * rho * (vx * vx + vy * vy + vz * vz)),
                                      P.f_smallp);
                const float cs = sqrtf(g * p * rhoinv);
                const float dtx = __fdividef(A.dx_f[0], fabsf(vx) + cs);
                const float dty = __fdividef(A.dx_f[1], fabsf(vy) + cs);
                const float dtz = __fdividef(A.dx_f[2], fabsf(vz) + cs);
                v = f2d_bits(fminf(dtx, fminf(dty, dtz)));
            } else {
                v = cfl_bound(P, un, A.dx);
            }
            local_dt = v < local_dt ? v : local_dt;
        }
    }
    if (A.cfl_min) block_min_atomic(local_dt, A.cfl_min);
}

ocfd_status configure_eb_tile() {
    if (cudaFuncSetAttribute(k_ebl_tile<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)ebt_smem_bytes<false>()) != cudaSuccess ||
        cudaFuncSetAttribute(k_ebl_tile<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)ebt_smem_bytes<true>()) != cudaSuccess)
        return check_launch("configure cut-cell tile kernel");
    return OCFD_OK;
}

}  // namespace ocfd

// ------------------------------------------------------------------ host side
struct ocfd::EbLevel {
    ocfd_eb_desc desc{};
    std::vector<int> cls;       // per box
    std::vector<int> geo_of;    // per box: geometry tag, or -1
    std::vector<GeoTag> geo;    // host copies of the geometry tags
    double* d_geo = nullptr;
    uint32_t* d_flag = nullptr;
    // cut and covered boxes (level box indices)
    std::vector<int> ebox;
    EbStageBox* d_stage[NUM_STAGE_SLOTS] = {nullptr, nullptr, nullptr, nullptr};
    bool cfl_slot[NUM_STAGE_SLOTS] = {false, false, true, false};  // fused CFL bound per stage slot
    // fused tile kernel: first tile of each cut / covered box (device) and the
    // tiles of each box (host, per-box launches), tiles in total; d_zero: a 0
    int* d_tstart = nullptr;
    int* d_zero = nullptr;
    std::vector<int> tcount;
    int ntiles = 0;
};

namespace ocfd {

static void eb_free_tables(ocfd_level* L) {
    EbLevel* E = L->eb;
    for (int s = 0; s < NUM_STAGE_SLOTS; ++s) {
        dev_free(E->d_stage[s], L->pool);
        E->d_stage[s] = nullptr;
    }
    dev_free(E->d_tstart, L->pool);
    dev_free(E->d_zero, L->pool);
    E->d_tstart = nullptr;
    E->d_zero = nullptr;
    E->ntiles = 0;
}

void eb_free(ocfd_level* L) {
    if (!L || !L->eb) return;
    EbLevel* E = L->eb;
    eb_free_tables(L);
    dev_free(E->d_geo, L->pool);
    dev_free(E->d_flag, L->pool);
    delete E;
    L->eb = nullptr;
}

bool eb_box_regular(const ocfd_level* L, int b) { return !L->eb || L->eb->cls[b] == OCFD_BOX_REGULAR; }
int eb_box_class(const ocfd_level* L, int b) { return L->eb ? L->eb->cls[b] : OCFD_BOX_REGULAR; }

const uint32_t* eb_box_flag(const ocfd_level* L, int b) {
    if (!L->eb || L->eb->geo_of[b] < 0 || L->eb->cls[b] != OCFD_BOX_CUT) return nullptr;
    return L->eb->d_flag + L->eb->geo[L->eb->geo_of[b]].off_fl;
}

bool eb_box_views(const ocfd_level* L, int b, View<const uint32_t>& flag, View<const double>& vfrac,
                  View<const double> ap[3]) {
    if (!L->eb || L->eb->geo_of[b] < 0 || L->eb->cls[b] != OCFD_BOX_CUT) return false;
    const EbLevel* E = L->eb;
    const GeoTag& g = E->geo[E->geo_of[b]];
    const int b0 = g.lo[0], b1 = g.lo[1];
    flag = View<const uint32_t>{E->d_flag + g.off_fl, g.gx, 0, 0, b0, b1, 0};
    vfrac = View<const double>{E->d_geo + g.off_vf, g.gx, 0, 0, b0, b1, 0};
    ap[0] = View<const double>{E->d_geo + g.off_ax, g.gx + 1, 0, 0, b0, b1, 0};
    ap[1] = View<const double>{E->d_geo + g.off_ay, g.gx, 0, 0, b0, b1, 0};
    ap[2] = vfrac;  // bodies extruded along z: the z faces' area fraction is the cell's volume fraction
    return true;
}

const double* eb_box_vfrac(const ocfd_level* L, int b, int* gx) {
    if (!L->eb || L->eb->geo_of[b] < 0 || L->eb->cls[b] != OCFD_BOX_CUT) return nullptr;
    const GeoTag& g = L->eb->geo[L->eb->geo_of[b]];
    if (gx) *gx = g.gx;
    return L->eb->d_geo + g.off_vf;
}

// squared distance bounds from (cx, cy) to the rectangle [x0, x1] x [y0, y1]
static void rect_dist2(double cx, double cy, double x0, double x1, double y0, double y1, double& dmin2,
                       double& dmax2) {
    const double ex = cx < x0 ? x0 - cx : (cx > x1 ? cx - x1 : 0.0);
    const double ey = cy < y0 ? y0 - cy : (cy > y1 ? cy - y1 : 0.0);
    dmin2 = ex * ex + ey * ey;
    const double fx = std::max(std::fabs(cx - x0), std::fabs(cx - x1));
    const double fy = std::max(std::fabs(cy - y0), std::fabs(cy - y1));
    dmax2 = fx * fx + fy * fy;
}

ocfd_status eb_setup(ocfd_level* L, const ocfd_eb_desc& eb) {
    eb_free(L);
    L->zvirt = L->zvirt_allowed;
    if (eb.kind == OCFD_EB_NONE) return OCFD_OK;
    if (eb.kind != OCFD_EB_CYLINDER_Z) return fail(OCFD_BAD_ARG, "ocfd_level_set_eb: unknown body kind");
    if (!(eb.radius > 0) || eb.nsub < 0 || eb.nsub > 256) return fail(OCFD_BAD_ARG, "ocfd_level_set_eb: radius / nsub");
    EbLevel* E = new EbLevel();
    L->eb = E;
    E->desc = eb;
    if (E->desc.nsub == 0) E->desc.nsub = 16;
    const int nb = (int)L->boxes.size();
    E->cls.assign(nb, OCFD_BOX_REGULAR);
    E->geo_of.assign(nb, -1);
    const double* plo = L->desc.prob_lo;
    const double* dx = L->desc.dx;
    const double r = eb.radius, r2 = r * r;
    // analytic screening: every sample point of grow(bx, 5) outside the circle ->
    // regular; every sample of bx inside -> covered; otherwise build the geometry
    std::map<std::tuple<int, int, int, int>, int> geo_index;
    long long nvf = 0, nfl = 0;
    for (int b = 0; b < nb; ++b) {
        const ocfd_box& B = L->boxes[b];
        double dmin2, dmax2;
        rect_dist2(eb.center[0], eb.center[1], plo[0] + (B.lo[0] - EB_GG) * dx[0], plo[0] + (B.hi[0] + 1 + EB_GG) * dx[0],
                   plo[1] + (B.lo[1] - EB_GG) * dx[1], plo[1] + (B.hi[1] + 1 + EB_GG) * dx[1], dmin2, dmax2);
        if (dmin2 > r2 * (1.0 + 1e-9) + 1e-300) continue;  // regular
        rect_dist2(eb.center[0], eb.center[1], plo[0] + B.lo[0] * dx[0], plo[0] + (B.hi[0] + 1) * dx[0],
                   plo[1] + B.lo[1] * dx[1], plo[1] + (B.hi[1] + 1) * dx[1], dmin2, dmax2);
        if (dmax2 < r2 * (1.0 - 1e-9)) {
            E->cls[b] = OCFD_BOX_COVERED;
            continue;
        }
        auto key = std::make_tuple(B.lo[0], B.lo[1], B.hi[0], B.hi[1]);
        auto it = geo_index.find(key);
        if (it != geo_index.end()) {
            E->geo_of[b] = it->second;
            continue;
        }
        GeoTag g{};
        g.lo[0] = B.lo[0] - EB_GG;
        g.lo[1] = B.lo[1] - EB_GG;
        g.gx = B.hi[0] - B.lo[0] + 1 + 2 * EB_GG;
        g.gy = B.hi[1] - B.lo[1] + 1 + 2 * EB_GG;
        g.off_vf = nvf;
        g.off_ax = g.off_vf + (long long)g.gx * g.gy;
        g.off_ay = g.off_ax + (long long)(g.gx + 1) * g.gy;
        nvf = g.off_ay + (long long)g.gx * (g.gy + 1);
        g.off_fl = nfl;
        nfl += (long long)g.gx * g.gy;
        const int id = (int)E->geo.size();
        E->geo.push_back(g);
        geo_index[key] = id;
        E->geo_of[b] = id;
    }
    const int ng = (int)E->geo.size();
    ocfd_status s = OCFD_OK;
    std::vector<unsigned long long> counts(2 * (size_t)std::max(ng, 1), 0ull);
    if (ng > 0) {
        E->d_geo = static_cast<double*>(dev_alloc(sizeof(double) * nvf, L->pool));
        E->d_flag = static_cast<uint32_t*>(dev_alloc(sizeof(uint32_t) * nfl, L->pool));
        if (!E->d_geo || !E->d_flag) return fail(OCFD_OUT_OF_MEMORY, "ocfd_level_set_eb: geometry");
        std::vector<long long> fstart(ng), cstart(ng);
        long long ftot = 0, ctot = 0;
        for (int g = 0; g < ng; ++g) {
            fstart[g] = ftot;
            ftot += (long long)(E->geo[g].gx + 1) * (E->geo[g].gy + 1);
            cstart[g] = ctot;
            ctot += (long long)E->geo[g].gx * E->geo[g].gy;
        }
        GeoTag* d_tags = nullptr;
        long long *d_fs = nullptr, *d_cs = nullptr;
        unsigned long long* d_counts = nullptr;
        s = upload(&d_tags, E->geo);
        if (s == OCFD_OK) s = upload(&d_fs, fstart);
        if (s == OCFD_OK) s = upload(&d_cs, cstart);
        if (s == OCFD_OK) s = upload(&d_counts, counts);
        if (s == OCFD_OK) {
            EbShape sh{};
            sh.kind = eb.kind;
            sh.nsub = E->desc.nsub;
            sh.cx = eb.center[0];
            sh.cy = eb.center[1];
            sh.r = eb.radius;
            for (int d = 0; d < 2; ++d) {
                sh.plo[d] = plo[d];
                sh.dx[d] = dx[d];
            }
            const int sms = L->ctx->num_sms;
            k_geom_frac<<<grid_for(ftot, 128, sms), 128>>>(d_tags, d_fs, ng, ftot, sh, E->d_geo);
            k_geom_flag<<<grid_for(ctot, 256, sms), 256>>>(d_tags, d_cs, ng, ctot, E->d_geo, E->d_flag, d_counts);
            s = check_launch("ocfd_level_set_eb geometry");
        }
        if (s == OCFD_OK && cudaMemcpy(counts.data(), d_counts, sizeof(unsigned long long) * 2 * ng,
                                       cudaMemcpyDeviceToHost) != cudaSuccess)
            s = fail(OCFD_LAUNCH_FAIL, "ocfd_level_set_eb: class counts");
        cudaFree(d_tags);
        cudaFree(d_fs);
        cudaFree(d_cs);
        cudaFree(d_counts);
        if (s != OCFD_OK) return s;
    }
    for (int b = 0; b < nb; ++b) {
        const int g = E->geo_of[b];
        if (g < 0) continue;
        const ocfd_box& B = L->boxes[b];
        const long long ncell_xy = (long long)(B.hi[0] - B.lo[0] + 1) * (B.hi[1] - B.lo[1] + 1);
        if (counts[2 * g + 1] == (unsigned long long)ncell_xy) E->cls[b] = OCFD_BOX_COVERED;
        else if (counts[2 * g] == 0) E->cls[b] = OCFD_BOX_REGULAR;
        else E->cls[b] = OCFD_BOX_CUT;
    }
    // the cut and covered boxes, in level order
    bool any_cut = false;
    for (int b = 0; b < nb; ++b) {
        if (E->cls[b] == OCFD_BOX_REGULAR) continue;
        E->ebox.push_back(b);
        if (E->cls[b] == OCFD_BOX_CUT) any_cut = true;
    }
    // the cut-cell stencils read z ghost cells from the state: fill them
    L->zvirt = L->zvirt_allowed && !any_cut;
    return OCFD_OK;
}

static ocfd_array4 fab_view(const ocfd_level* L, int b, int i) {
    const FabGeom& f = L->fabs[b];
    ocfd_array4 a{};
    a.p = L->buf[i] + f.off;
    a.jstride = f.g[0];
    a.kstride = (long long)f.g[0] * f.g[1];
    a.nstride = f.ns;
    for (int d = 0; d < 3; ++d) {
        a.begin[d] = f.lo[d] - NGR;
        a.end[d] = f.hi[d] + NGR + 1;
    }
    a.ncomp = L->ncomp;
    return a;
}

ocfd_status eb_build_stage_tables(ocfd_level* L, const StageRoles& roles) {
    EbLevel* E = L->eb;
    if (!E) return OCFD_OK;
    eb_free_tables(L);
    const int ne = (int)E->ebox.size();
    if (ne == 0) return OCFD_OK;
    StageSlot slot[NUM_STAGE_SLOTS];
    for (int k = 0; k < NUM_STAGE_SLOTS; ++k) {
        slot[k] = stage_slot(L->rk_order, roles, k);
        E->cfl_slot[k] = slot[k].cfl;
    }
    std::vector<EbStageBox> st[NUM_STAGE_SLOTS];
    std::vector<int> ts(ne);
    int tt = 0;
    E->tcount.assign(ne, 0);
    for (int e = 0; e < ne; ++e) {
        const int b = E->ebox[e];
        const ocfd_box& B = L->boxes[b];
        const int n[3] = {B.hi[0] - B.lo[0] + 1, B.hi[1] - B.lo[1] + 1, B.hi[2] - B.lo[2] + 1};
        const bool cut = E->cls[b] == OCFD_BOX_CUT;
        ts[e] = tt;
        E->tcount[e] = ((n[0] + EBT_X - 1) / EBT_X) * ((n[1] + EBT_Y - 1) / EBT_Y) * ((n[2] + EBT_Z - 1) / EBT_Z);
        tt += E->tcount[e];
        EbStageBox base{};
        for (int d = 0; d < 3; ++d) {
            base.lo[d] = B.lo[d];
            base.hi[d] = B.hi[d];
        }
        base.covered = cut ? 0 : 1;
        if (cut) {
            const GeoTag& g = E->geo[E->geo_of[b]];
            const int b0 = g.lo[0], b1 = g.lo[1];
            base.flag = View<const uint32_t>{E->d_flag + g.off_fl, g.gx, 0, 0, b0, b1, 0};
            base.vfrac = View<const double>{E->d_geo + g.off_vf, g.gx, 0, 0, b0, b1, 0};
            base.ap[0] = View<const double>{E->d_geo + g.off_ax, g.gx + 1, 0, 0, b0, b1, 0};
            base.ap[1] = View<const double>{E->d_geo + g.off_ay, g.gx, 0, 0, b0, b1, 0};
            base.ap[2] = base.vfrac;
        }
        if (!roles.flux_bits.empty() && roles.flux_bits[b] && cut) {
            base.has_flux = roles.flux_bits[b] & (FLUX_ACC_ALL | FLUX_ACC_PLANES);
            if (base.has_flux & FLUX_ACC_ALL)
                for (int d = 0; d < 3; ++d) base.creg[d] = roles.creg[3 * b + d];
            if (base.has_flux & FLUX_ACC_PLANES)
                for (int d = 0; d < 3; ++d)
                    for (int sd = 0; sd < 2; ++sd) base.fplane[d][sd] = roles.fplane[6 * b + 2 * d + sd];
        }
        ocfd_array4 a[4];
        for (int i = 0; i < L->nbuf; ++i) a[i] = fab_view(L, b, i);
        for (int k = 0; k < NUM_STAGE_SLOTS; ++k) {
            if (!slot[k].used) continue;
            EbStageBox x = base;
            x.S = view_of<const double>(&a[slot[k].src]);
            x.U0 = view_of<const double>(&a[0]);
            x.Uout = view_of<double>(&a[slot[k].out]);
            x.rk_a = slot[k].a;
            x.rk_b = slot[k].b;
            x.flux_w = slot[k].w;
            st[k].push_back(x);
        }
    }
    E->ntiles = tt;
    ocfd_status s = OCFD_OK;
    for (int k = 0; k < NUM_STAGE_SLOTS && s == OCFD_OK; ++k) s = upload(&E->d_stage[k], st[k], L->pool);
    if (s == OCFD_OK) s = upload(&E->d_tstart, ts, L->pool);
    if (s == OCFD_OK) s = upload(&E->d_zero, std::vector<int>(1, 0), L->pool);
    return s;
}

ocfd_status eb_launch_stage(ocfd_level* L, int s, unsigned flags, cudaStream_t st) {
    EbLevel* E = L->eb;
    if (!E || E->ebox.empty() || E->ntiles == 0) return OCFD_OK;
    EbStageArgs A{};
    A.boxes = E->d_stage[s];
    A.nbox = (int)E->ebox.size();
    for (int d = 0; d < 3; ++d) {
        A.dxinv[d] = 1.0 / L->desc.dx[d];
        A.dx[d] = L->desc.dx[d];
        A.dxinv_f[d] = (float)A.dxinv[d];
        A.dx_f[d] = (float)L->desc.dx[d];
    }
    A.dt_ptr = &L->d_step->dt;
    A.cfl_min = E->cfl_slot[s] ? &L->d_step->cfl_min : nullptr;
    A.visc = (flags & OCFD_VISC) ? 1 : 0;
    A.redist = E->desc.redistribute ? 1 : 0;
    const bool f32 = (flags & OCFD_FLUX_FP32) && !A.visc;
    auto go = [&](const EbStageArgs& X, const int* tstart, int ntiles) {
        if (f32) k_ebl_tile<true><<<ntiles, EBT_N, ebt_smem_bytes<true>(A.visc), st>>>(X, tstart, L->ctx->parm);
        else k_ebl_tile<false><<<ntiles, EBT_N, ebt_smem_bytes<false>(A.visc), st>>>(X, tstart, L->ctx->parm);
    };
    if (flags & OCFD_PER_BOX) {
        // one launch per box (the reference's per-box execution model), the same kernel
        for (int e = 0; e < (int)E->ebox.size(); ++e) {
            EbStageArgs B = A;
            B.boxes = E->d_stage[s] + e;
            B.nbox = 1;
            go(B, E->d_zero, E->tcount[e]);
        }
        return check_launch("level cut-cell stage (per box)");
    }
    // batched: every cut and covered box of the level in one launch
    go(A, E->d_tstart, E->ntiles);
    return check_launch("level cut-cell stage");
}

int eb_launches_per_stage(const ocfd_level* L, unsigned flags) {
    const EbLevel* E = L->eb;
    if (!E || E->ebox.empty()) return 0;
    if (flags & OCFD_PER_BOX) return (int)E->ebox.size();
    return E->ntiles > 0 ? 1 : 0;
}

}  // namespace ocfd

using namespace ocfd;

extern "C" {

ocfd_status ocfd_level_set_eb(ocfd_level* L, const ocfd_eb_desc* eb) {
    if (!L || !eb) return fail(OCFD_BAD_ARG, "ocfd_level_set_eb: null argument");
    if (L->ncomp != 5) return fail(OCFD_BAD_ARG, "ocfd_level_set_eb: the cut-cell level path is the ideal-gas one");
    if (cudaDeviceSynchronize() != cudaSuccess) return check_launch("ocfd_level_set_eb");
    ocfd_status s = eb_setup(L, *eb);
    if (s == OCFD_OK) s = rebuild_fill_tags(L);
    if (s == OCFD_OK) s = build_stage_tables(L, StageRoles{});
    if (s == OCFD_OK && cudaDeviceSynchronize() != cudaSuccess) s = fail(OCFD_LAUNCH_FAIL, "ocfd_level_set_eb");
    if (L->graph) {
        cudaGraphExecDestroy(L->graph);
        L->graph = nullptr;
    }
    return s;
}

ocfd_status ocfd_level_box_classes(const ocfd_level* L, int32_t* classes) {
    if (!L || !classes) return fail(OCFD_BAD_ARG, "ocfd_level_box_classes");
    for (int b = 0; b < (int)L->boxes.size(); ++b) classes[b] = eb_box_class(L, b);
    return OCFD_OK;
}

ocfd_status ocfd_level_eb_geometry(const ocfd_level* L, int ibox, ocfd_flag4* flag, ocfd_array4* vfrac,
                                   ocfd_array4* ap) {
    if (!L || ibox < 0 || ibox >= (int)L->boxes.size() || !flag || !vfrac || !ap)
        return fail(OCFD_BAD_ARG, "ocfd_level_eb_geometry");
    const EbLevel* E = L->eb;
    if (!E || E->geo_of[ibox] < 0) return fail(OCFD_BAD_ARG, "ocfd_level_eb_geometry: box has no cut-cell data");
    const GeoTag& g = E->geo[E->geo_of[ibox]];
    const ocfd_box& B = L->boxes[ibox];
    auto fill = [&](int64_t js, int nxe, int nye, int32_t* begin, int32_t* end) {
        begin[0] = g.lo[0];
        begin[1] = g.lo[1];
        begin[2] = B.lo[2] - EB_GG;
        end[0] = g.lo[0] + nxe;
        end[1] = g.lo[1] + nye;
        end[2] = B.hi[2] + EB_GG + 1;
        (void)js;
    };
    flag->p = E->d_flag + g.off_fl;
    flag->jstride = g.gx;
    flag->kstride = 0;
    flag->nstride = 0;
    flag->ncomp = 1;
    fill(g.gx, g.gx, g.gy, flag->begin, flag->end);
    *vfrac = ocfd_array4{E->d_geo + g.off_vf, g.gx, 0, 0, {0, 0, 0}, {0, 0, 0}, 1};
    fill(g.gx, g.gx, g.gy, vfrac->begin, vfrac->end);
    ap[0] = ocfd_array4{E->d_geo + g.off_ax, g.gx + 1, 0, 0, {0, 0, 0}, {0, 0, 0}, 1};
    fill(g.gx + 1, g.gx + 1, g.gy, ap[0].begin, ap[0].end);
    ap[1] = ocfd_array4{E->d_geo + g.off_ay, g.gx, 0, 0, {0, 0, 0}, {0, 0, 0}, 1};
    fill(g.gx, g.gx, g.gy + 1, ap[1].begin, ap[1].end);
    ap[2] = *vfrac;
    ap[2].end[2] += 1;
    return OCFD_OK;
}

ocfd_status ocfd_level_eb_geometry_copy(const ocfd_level* L, int ibox, uint32_t* flag, double* vfrac,
                                        double* apx, double* apy) {
    if (!L || ibox < 0 || ibox >= (int)L->boxes.size() || !flag || !vfrac || !apx || !apy)
        return fail(OCFD_BAD_ARG, "ocfd_level_eb_geometry_copy");
    const EbLevel* E = L->eb;
    if (!E || E->geo_of[ibox] < 0) return fail(OCFD_BAD_ARG, "ocfd_level_eb_geometry_copy: box has no cut-cell data");
    const GeoTag& g = E->geo[E->geo_of[ibox]];
    const size_t nc = (size_t)g.gx * g.gy;
    bool ok = cudaMemcpy(flag, E->d_flag + g.off_fl, sizeof(uint32_t) * nc, cudaMemcpyDeviceToHost) == cudaSuccess &&
              cudaMemcpy(vfrac, E->d_geo + g.off_vf, sizeof(double) * nc, cudaMemcpyDeviceToHost) == cudaSuccess &&
              cudaMemcpy(apx, E->d_geo + g.off_ax, sizeof(double) * (g.gx + 1) * g.gy, cudaMemcpyDeviceToHost) ==
                  cudaSuccess &&
              cudaMemcpy(apy, E->d_geo + g.off_ay, sizeof(double) * g.gx * (g.gy + 1), cudaMemcpyDeviceToHost) ==
                  cudaSuccess;
    return ok ? OCFD_OK : fail(OCFD_LAUNCH_FAIL, "ocfd_level_eb_geometry_copy");
}

}  // extern "C"
