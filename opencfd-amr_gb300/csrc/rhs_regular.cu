// Fused right-hand side of a regular (uncut) box, ideal gas, FP64.
//
// Replaces the per-box kernel chain of EBR::compute_dSdt (Source/Advance.cpp:
// 231-329): c2prim over the grown box, then per direction flux_split (full
// grown box), reconstruction (WENO-Z, per face and component), compute_visc,
// and finally divop.  Here one CTA owns a TX x TY x TZ tile of the box and
// never writes an intermediate to HBM:
//
//   per direction D:
//     1. the tile's pencil along D (tile + 3 cells each side) is read from the
//        state, turned into primitives and split into F+ / F- (10 values per
//        cell) in shared memory,
//     2. WENO-Z face fluxes of the tile's T_D+1 faces x 5 components are formed
//        in shared memory (work items = face x component),
//     3. with OCFD_VISC the viscous stress / heat flux is added per face from
//        a primitive ring (tile grown by 1) staged once per tile,
//     4. each cell thread accumulates dxinv_D (F_f - F_f+1) in registers, in the
//        reference's summation order x, y, z (Source/kernel/Kernels.H:94-96);
//        face fluxes are written out when the caller asked for them (reflux).
//   Only U (read) and dSdt (write) touch HBM: 80 B per cell, plus halo re-reads
//   that hit L2.
#include <cuda_runtime.h>

#include "device_physics.cuh"
#include "ocfd_internal.h"
#include "rhs_regular.h"

namespace ocfd {

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
    static constexpr int SMEM = 10 * N + 5 * NF;                       // doubles
};

template <int TX, int TY, int TZ>
struct Ring {
    static constexpr int RX = TX + 2, RY = TY + 2, RZ = TZ + 2;
    static constexpr int N = RX * RY * RZ;
};

template <int TX, int TY, int TZ, bool VISC>
__host__ __device__ constexpr int regular_smem_doubles() {
    constexpr int a = Pencil<0, TX, TY, TZ>::SMEM;
    constexpr int b = Pencil<1, TX, TY, TZ>::SMEM;
    constexpr int c = Pencil<2, TX, TY, TZ>::SMEM;
    constexpr int m = a > b ? (a > c ? a : c) : (b > c ? b : c);
    return m + (VISC ? 4 * Ring<TX, TY, TZ>::N : 0);
}

constexpr size_t kMaxSmem = 227 * 1024;  // opt-in dynamic shared memory per CTA

// Viscous stress and heat flux of the D-face between ring cells (r - e_D) and r,
// Source/kernel/Diffusion.H:7-131.  ring holds u, v, w, T (4 planes of RN).
template <int D, int TX, int TY, int TZ>
__device__ __forceinline__ void visc_face(const DevParm& P, const double* ring, int rx, int ry,
                                          int rz, const double* dxinv, double* f /*stride fs*/,
                                          int fs) {
    using R = Ring<TX, TY, TZ>;
    constexpr int S[3] = {1, R::RX, R::RX * R::RY};
    const int c = rx + ry * R::RX + rz * R::RX * R::RY;
    const int l = c - S[D];
    const double* qu = ring;
    const double* qT = ring + 3 * R::N;
    double Tr = qT[c], Tl = qT[l];
    double mutl = sutherland(P, Tl), mutr = sutherland(P, Tr);
    double ktl = mutl * P.kOverMu, ktr = mutr * P.kOverMu;
    double dT = (Tr - Tl) * dxinv[D];
    double g[3][3];
#pragma unroll
    for (int m = 0; m < 3; ++m) g[m][D] = (qu[m * R::N + c] - qu[m * R::N + l]) * dxinv[D];
#pragma unroll
    for (int t = 0; t < 3; ++t) {
        if (t == D) continue;
        const int st = S[t];
        // d(u_D)/dx_t and d(u_t)/dx_t averaged over the two cells of the face
        g[D][t] = (qu[D * R::N + c + st] + qu[D * R::N + l + st] - qu[D * R::N + c - st] -
                   qu[D * R::N + l - st]) * (0.25 * dxinv[t]);
        g[t][t] = (qu[t * R::N + c + st] + qu[t * R::N + l + st] - qu[t * R::N + c - st] -
                   qu[t * R::N + l - st]) * (0.25 * dxinv[t]);
    }
    double divu = g[0][0] + g[1][1] + g[2][2];
    double muf = 0.5 * (mutl + mutr);
    double tau[3];
#pragma unroll
    for (int m = 0; m < 3; ++m)
        tau[m] = (m == D) ? muf * (2.0 * g[D][D] - P.twoThirds * divu) : muf * (g[m][D] + g[D][m]);
#pragma unroll
    for (int m = 0; m < 3; ++m) f[(1 + m) * fs] += -tau[m];
    f[4 * fs] += -0.5 * ((qu[c] + qu[l]) * tau[0] + (qu[R::N + c] + qu[R::N + l]) * tau[1] +
                         (qu[2 * R::N + c] + qu[2 * R::N + l]) * tau[2] + (ktl + ktr) * dT);
}

template <int D, int TX, int TY, int TZ, bool VISC>
__device__ __forceinline__ void sweep(const RegBoxArgs& B, const DevParm& P, int i0, int j0, int k0,
                                      double* F, double* FF, const double* ring, double* acc) {
    using PC = Pencil<D, TX, TY, TZ>;
    constexpr int NT = TX * TY * TZ;
    const int tid = threadIdx.x;
    const int org[3] = {i0, j0, k0};
    // ---- 1. primitives and Steger-Warming split over the pencil
    for (int c = tid; c < PC::N; c += NT) {
        const int px = c % PC::PX, py = (c / PC::PX) % PC::PY, pz = c / (PC::PX * PC::PY);
        const int gi = i0 + px - (D == 0 ? 3 : 0);
        const int gj = j0 + py - (D == 1 ? 3 : 0);
        const int gk = k0 + pz - (D == 2 ? 3 : 0);
        double fp[5] = {0, 0, 0, 0, 0}, fm[5] = {0, 0, 0, 0, 0};
        if (gi <= B.hi[0] + (D == 0 ? 3 : 0) && gj <= B.hi[1] + (D == 1 ? 3 : 0) &&
            gk <= B.hi[2] + (D == 2 ? 3 : 0)) {
            double q[7];
            c2prim_ideal(P, B.S(gi, gj, gk, 0), B.S(gi, gj, gk, 1), B.S(gi, gj, gk, 2),
                         B.S(gi, gj, gk, 3), B.S(gi, gj, gk, 4), q);
            sw_split<D>(q[QRHO], q[QU], q[QV], q[QW], q[QC], P.sw_tmp1, P.sw_tmp2, P.sw_tmp3,
                        P.sw_gm1, fp, fm);
        }
#pragma unroll
        for (int n = 0; n < 5; ++n) {
            F[n * PC::N + c] = fp[n];
            F[(5 + n) * PC::N + c] = fm[n];
        }
    }
    __syncthreads();
    // ---- 2. WENO-Z face fluxes
    for (int it = tid; it < 5 * PC::NF; it += NT) {
        const int n = it / PC::NF, f = it - n * PC::NF;
        const int fx = f % PC::FX, fy = (f / PC::FX) % PC::FY, fz = f / (PC::FX * PC::FY);
        const int base = fx + fy * PC::PX + fz * PC::PX * PC::PY;
        const double* a = F + n * PC::N + base;
        const double* b = F + (5 + n) * PC::N + base;
        constexpr int s = PC::PST;
        FF[n * PC::NF + f] = wenoz_plus(a[0], a[s], a[2 * s], a[3 * s], a[4 * s]) +
                             wenoz_minus(b[s], b[2 * s], b[3 * s], b[4 * s], b[5 * s]);
    }
    __syncthreads();
    // ---- 3. viscous part of the face flux
    if (VISC) {
        for (int f = tid; f < PC::NF; f += NT) {
            const int fx = f % PC::FX, fy = (f / PC::FX) % PC::FY, fz = f / (PC::FX * PC::FY);
            // ring coordinates of the cell on the high side of the face
            visc_face<D, TX, TY, TZ>(P, ring, fx + 1, fy + 1, fz + 1, B.dxinv, FF + f, PC::NF);
        }
        __syncthreads();
    }
    // ---- 4. divergence contribution and optional face-flux output
    {
        const int ti = tid % TX, tj = (tid / TX) % TY, tk = tid / (TX * TY);
        const int f = ti + tj * PC::FX + tk * PC::FX * PC::FY;
#pragma unroll
        for (int n = 0; n < 5; ++n) {
            double v = B.dxinv[D] * (FF[n * PC::NF + f] - FF[n * PC::NF + f + PC::FST]);
            acc[n] = (D == 0) ? v : acc[n] + v;
        }
    }
    if (B.has_flux) {
        const View<double>& out = B.flux[D];
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
#pragma unroll
                for (int n = 0; n < 5; ++n) out(gi, gj, gk, n) = FF[n * PC::NF + f];
            }
        }
    }
    (void)org;
    __syncthreads();
}

template <int TX, int TY, int TZ, bool VISC>
__global__ void __launch_bounds__(TX* TY* TZ)
    k_rhs_regular(const RegBoxArgs* __restrict__ boxes, const int* __restrict__ tile_start,
                  int nbox, RegBoxArgs single, DevParm P) {
    extern __shared__ double smem[];
    constexpr int NT = TX * TY * TZ;
    // locate the box of this CTA: a single box, or a prefix table over a box list
    int b = 0;
    int t = blockIdx.x;
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

    constexpr int PMAX = regular_smem_doubles<TX, TY, TZ, false>();
    double* F = smem;
    double* ring = smem + PMAX;
    if (VISC) {
        using R = Ring<TX, TY, TZ>;
        for (int c = threadIdx.x; c < R::N; c += NT) {
            const int rx = c % R::RX, ry = (c / R::RX) % R::RY, rz = c / (R::RX * R::RY);
            const int gi = i0 + rx - 1, gj = j0 + ry - 1, gk = k0 + rz - 1;
            double q[7] = {0, 0, 0, 0, 0, 1, 0};
            if (gi <= B.hi[0] + 1 && gj <= B.hi[1] + 1 && gk <= B.hi[2] + 1)
                c2prim_ideal(P, B.S(gi, gj, gk, 0), B.S(gi, gj, gk, 1), B.S(gi, gj, gk, 2),
                             B.S(gi, gj, gk, 3), B.S(gi, gj, gk, 4), q);
            ring[c] = q[QU];
            ring[R::N + c] = q[QV];
            ring[2 * R::N + c] = q[QW];
            ring[3 * R::N + c] = q[QT];
        }
        __syncthreads();
    }
    double acc[5];
    sweep<0, TX, TY, TZ, VISC>(B, P, i0, j0, k0, F, F + 10 * Pencil<0, TX, TY, TZ>::N, ring, acc);
    sweep<1, TX, TY, TZ, VISC>(B, P, i0, j0, k0, F, F + 10 * Pencil<1, TX, TY, TZ>::N, ring, acc);
    sweep<2, TX, TY, TZ, VISC>(B, P, i0, j0, k0, F, F + 10 * Pencil<2, TX, TY, TZ>::N, ring, acc);

    const int ti = threadIdx.x % TX, tj = (threadIdx.x / TX) % TY, tk = threadIdx.x / (TX * TY);
    const int ci = i0 + ti, cj = j0 + tj, ck = k0 + tk;
    const bool valid = ci <= B.hi[0] && cj <= B.hi[1] && ck <= B.hi[2];
    double local_dt = __longlong_as_double(0x7FF0000000000000LL);
    if (valid) {
        if (B.mode == RHS_WRITE_DSDT) {
#pragma unroll
            for (int n = 0; n < 5; ++n) B.dsdt(ci, cj, ck, n) = acc[n];
        } else {
            // fused Shu-Osher stage: U_out = a U0 + b (U_s + dt L(U_s))
            const double dt = B.dt_ptr ? *B.dt_ptr : B.dt;
            double un[5];
#pragma unroll
            for (int n = 0; n < 5; ++n) {
                double us = B.S(ci, cj, ck, n);
                double u0 = B.U0(ci, cj, ck, n);
                un[n] = B.rk_a * u0 + B.rk_b * (us + dt * acc[n]);
                B.Uout(ci, cj, ck, n) = un[n];
            }
            if (B.cfl_min) local_dt = cfl_bound(P, un, B.dx);
        }
    }
    if (B.cfl_min) block_min_atomic(local_dt, B.cfl_min);
}

template <int TX, int TY, int TZ, bool VISC>
static ocfd_status launch_t(const RegBoxArgs* d_boxes, const int* d_tile_start, int nbox,
                            const RegBoxArgs& single, int ntiles, const DevParm& P,
                            cudaStream_t st) {
    constexpr int NT = TX * TY * TZ;
    constexpr size_t smem = sizeof(double) * regular_smem_doubles<TX, TY, TZ, VISC>();
    auto kern = k_rhs_regular<TX, TY, TZ, VISC>;
    if (smem > kMaxSmem) return fail(OCFD_BAD_ARG, "regular RHS tile does not fit shared memory in this mode");
    if (ntiles <= 0) return OCFD_OK;
    kern<<<ntiles, NT, smem, st>>>(d_boxes, d_tile_start, nbox, single, P);
    return check_launch("k_rhs_regular");
}

template <int TX, int TY, int TZ, bool VISC>
static bool configure_one() {
    const size_t smem = sizeof(double) * regular_smem_doubles<TX, TY, TZ, VISC>();
    if (smem > kMaxSmem) return true;  // shape not offered in this mode
    return cudaFuncSetAttribute(k_rhs_regular<TX, TY, TZ, VISC>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess;
}

template <int TX, int TY, int TZ>
static bool configure_t() {
    return configure_one<TX, TY, TZ, false>() && configure_one<TX, TY, TZ, true>();
}

// Raises the dynamic shared-memory limit of every regular-RHS instantiation;
// called once per context, outside any stream capture.
ocfd_status configure_rhs_regular() {
    bool ok = configure_t<8, 8, 8>() && configure_t<8, 8, 4>() && configure_t<16, 8, 4>() &&
              configure_t<16, 16, 2>() && configure_t<32, 8, 2>() && configure_t<16, 8, 2>();
    if (!ok) return check_launch("configure_rhs_regular");
    return OCFD_OK;
}

template <int TX, int TY, int TZ>
static size_t smem_t(bool visc) {
    return visc ? sizeof(double) * regular_smem_doubles<TX, TY, TZ, true>()
                : sizeof(double) * regular_smem_doubles<TX, TY, TZ, false>();
}

bool regular_tile_fits(int tile, bool visc) {
    size_t b = 0;
    switch (tile) {
        case 0: b = smem_t<8, 8, 8>(visc); break;
        case 1: b = smem_t<8, 8, 4>(visc); break;
        case 2: b = smem_t<16, 8, 4>(visc); break;
        case 3: b = smem_t<16, 16, 2>(visc); break;
        case 4: b = smem_t<32, 8, 2>(visc); break;
        case 5: b = smem_t<16, 8, 2>(visc); break;
        default: return false;
    }
    return b <= kMaxSmem;
}

const TileShape kRegularTiles[] = {{8, 8, 8}, {8, 8, 4}, {16, 8, 4}, {16, 16, 2}, {32, 8, 2}, {16, 8, 2}};
const int kNumRegularTiles = sizeof(kRegularTiles) / sizeof(kRegularTiles[0]);

ocfd_status launch_rhs_regular(int tile, bool visc, const RegBoxArgs* d_boxes,
                               const int* d_tile_start, int nbox, const RegBoxArgs& single,
                               int ntiles, const DevParm& P, cudaStream_t st) {
#define OCFD_CASE(I, X, Y, Z)                                                                    \
    case I:                                                                                      \
        return visc ? launch_t<X, Y, Z, true>(d_boxes, d_tile_start, nbox, single, ntiles, P, st) \
                    : launch_t<X, Y, Z, false>(d_boxes, d_tile_start, nbox, single, ntiles, P, st);
    switch (tile) {
        OCFD_CASE(0, 8, 8, 8)
        OCFD_CASE(1, 8, 8, 4)
        OCFD_CASE(2, 16, 8, 4)
        OCFD_CASE(3, 16, 16, 2)
        OCFD_CASE(4, 32, 8, 2)
        OCFD_CASE(5, 16, 8, 2)
    }
#undef OCFD_CASE
    return fail(OCFD_BAD_ARG, "launch_rhs_regular: bad tile index");
}

// Default tile for a box: the shape with the least padded work.
int pick_regular_tile(const int n[3], bool visc) {
    int best = 1;
    double best_cost = 1e300;
    for (int t = 0; t < kNumRegularTiles; ++t) {
        if (!regular_tile_fits(t, visc)) continue;
        const TileShape& s = kRegularTiles[t];
        long long tiles = (long long)((n[0] + s.x - 1) / s.x) * ((n[1] + s.y - 1) / s.y) *
                          ((n[2] + s.z - 1) / s.z);
        // padded cells plus pencil halo work per tile (6 cells per direction)
        double per_tile = (double)s.x * s.y * s.z * 3.0 +
                          6.0 * ((double)s.y * s.z + (double)s.x * s.z + (double)s.x * s.y);
        double cost = tiles * per_tile;
        if (cost < best_cost * 0.999) {
            best_cost = cost;
            best = t;
        }
    }
    return best;
}

void fill_regular_args(RegBoxArgs& a, const ocfd_array4* S, const ocfd_array4* dSdt,
                       const ocfd_array4* flux, const ocfd_box& bx, const double dxinv[3],
                       int tile) {
    a.S = view_of<const double>(S);
    if (dSdt) a.dsdt = view_of<double>(dSdt);
    a.has_flux = flux != nullptr;
    for (int d = 0; d < 3; ++d) {
        if (flux) a.flux[d] = view_of<double>(&flux[d]);
        a.lo[d] = bx.lo[d];
        a.hi[d] = bx.hi[d];
        a.dxinv[d] = dxinv[d];
    }
    const TileShape& s = kRegularTiles[tile];
    const int T[3] = {s.x, s.y, s.z};
    for (int d = 0; d < 3; ++d) a.ntile[d] = (bx.hi[d] - bx.lo[d] + T[d]) / T[d];
    a.mode = RHS_WRITE_DSDT;
    a.dt_ptr = nullptr;
    a.cfl_min = nullptr;
}

}  // namespace ocfd

using namespace ocfd;

extern "C" ocfd_status ocfd_rhs_regular_box_f64(ocfd_context* ctx, const ocfd_array4* S,
                                                const ocfd_array4* dSdt, const ocfd_array4* flux,
                                                ocfd_box bx, const double dxinv[3],
                                                unsigned flags, void* stream) {
    if (!ctx || !dxinv) return fail(OCFD_BAD_ARG, "ocfd_rhs_regular_box_f64: null argument");
    for (int d = 0; d < 3; ++d)
        if (bx.hi[d] < bx.lo[d]) return fail(OCFD_BAD_ARG, "ocfd_rhs_regular_box_f64: empty box");
    if (!covers(S, bx, 3, 5)) return fail(OCFD_BAD_ARG, "ocfd_rhs_regular_box_f64: S must cover grow(bx,3) with 5 components");
    if (!covers(dSdt, bx, 0, 5)) return fail(OCFD_BAD_ARG, "ocfd_rhs_regular_box_f64: dSdt must cover bx with 5 components");
    if (flux)
        for (int d = 0; d < 3; ++d)
            if (!covers(&flux[d], bx, 0, 5, d))
                return fail(OCFD_BAD_ARG, "ocfd_rhs_regular_box_f64: flux[d] must cover surroundingNodes(bx,d)");
    if (flags & ~(unsigned)(OCFD_VISC | OCFD_FLUX_FP32))
        return fail(OCFD_BAD_ARG, "ocfd_rhs_regular_box_f64: unknown flags");
    if (flags & OCFD_FLUX_FP32) return rhs_regular_box_f32(ctx, S, dSdt, flux, bx, dxinv, flags, stream);
    const int n[3] = {bx.hi[0] - bx.lo[0] + 1, bx.hi[1] - bx.lo[1] + 1, bx.hi[2] - bx.lo[2] + 1};
    const int tile = pick_regular_tile(n, (flags & OCFD_VISC) != 0);
    RegBoxArgs a{};
    fill_regular_args(a, S, dSdt, flux, bx, dxinv, tile);
    const int ntiles = a.ntile[0] * a.ntile[1] * a.ntile[2];
    return launch_rhs_regular(tile, (flags & OCFD_VISC) != 0, nullptr, nullptr, 1, a, ntiles,
                              ctx->parm, static_cast<cudaStream_t>(stream));
}
