// AMR hierarchy on the GPU: subcycled SSP-RK3 (or RK2 / Euler: the rows of
// rk_scheme, coarse-fine ghosts then interpolated linearly in time between the
// coarse old and new states) over levels of ratio 2 with
// coarse-fine ghost interpolation (space and time), flux registers + reflux,
// average-down, CFL over all levels, density-gradient regridding.
//
// One coarse step (AMReX Amr::timeStep recursion, EBR::advance,
// EBR::post_timestep; Source/EBR.cpp:312-360) is captured as one CUDA graph:
//
//   k_amr_begin: dt_0 = cfl * min_l(est_l * 2^l) (1.1 dt_prev, stop time),
//                dt_l = dt_0 / 2^l
//   advance(0, 1)
//   estdt of every level (for the next step), k_amr_end: t += dt_0
//
//   advance(l, it):                        (it = 1..2 for l >= 1)
//     zero the coarse side of level l's flux register and the fine side of l+1's
//     stage s = 1..3:  ghosts of the stage input:
//                        coarse-fine cells interpolated from level l-1's RK3 stage
//                        states at the matching time (below), exchange, physical BCs
//                      fused RHS + Shu-Osher stage; RK3-weighted face fluxes
//                      accumulated into the flux registers
//     if level l+1 exists:
//        stage 3 writes buffer D (U^n stays in A), D's ghosts filled at t + dt_l
//        advance(l+1, 1); advance(l+1, 2)
//        reflux of the uncovered cells next to level l+1, average-down of the
//        covered cells, D -> A
//
// Time interpolation of coarse-fine ghosts.  From the coarse stage states
// u0 = A, U1 = B, U2 = C, U3 = D the scaled stage derivatives are
//   K1 = U1 - u0,  K2 = 4 U2 - 3 u0 - U1,  K3 = (3 U3 - u0 - 2 U2) / 2
// and the SSP-RK3 dense output at theta in [0, 1] of the coarse step is
//   P(theta) = u0 + (theta - 5/6 theta^2) K1 + theta^2/6 K2 + 2/3 theta^2 K3.
// A fine substep from theta to theta + r (r = 1/2) fills its three stages with
// the Taylor expansion of the fine stage states (u, u + h u', u + h/2 u' +
// h^2/4 u'' for SSP-RK3) evaluated on P, following McCorquodale & Colella,
// "A high-order finite-volume method for conservation laws on locally refined
// grids", CAMCoS 6 (2011), sec. 3.  Every value is a fixed linear combination
// a_A A + a_B B + a_C C + a_D D with sum(a) = 1, so the interpolation kernel
// mixes the four buffers and then applies MC-limited conservative linear
// slopes (van Leer) in space.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "host_sort.h"
#include "level.h"
#include "eb_level.h"
#include "chem_internal.h"

namespace ocfd {

// ================================================================ box algebra
struct IBox {
    int lo[3], hi[3];
};

static bool ib_empty(const IBox& b) {
    return b.lo[0] > b.hi[0] || b.lo[1] > b.hi[1] || b.lo[2] > b.hi[2];
}
static IBox ib_of(const ocfd_box& b) {
    IBox r;
    for (int d = 0; d < 3; ++d) { r.lo[d] = b.lo[d]; r.hi[d] = b.hi[d]; }
    return r;
}
static ocfd_box ob_of(const IBox& b) {
    ocfd_box r;
    for (int d = 0; d < 3; ++d) { r.lo[d] = b.lo[d]; r.hi[d] = b.hi[d]; }
    return r;
}
static bool ib_isect(const IBox& a, const IBox& b, IBox& o) {
    for (int d = 0; d < 3; ++d) {
        o.lo[d] = std::max(a.lo[d], b.lo[d]);
        o.hi[d] = std::min(a.hi[d], b.hi[d]);
        if (o.lo[d] > o.hi[d]) return false;
    }
    return true;
}
static IBox ib_grow(const IBox& b, int g) {
    IBox r = b;
    for (int d = 0; d < 3; ++d) { r.lo[d] -= g; r.hi[d] += g; }
    return r;
}
static int floordiv2(int x) { return x >= 0 ? x / 2 : -((1 - x) / 2); }
static IBox ib_coarsen(const IBox& b) {
    IBox r;
    for (int d = 0; d < 3; ++d) { r.lo[d] = floordiv2(b.lo[d]); r.hi[d] = floordiv2(b.hi[d]); }
    return r;
}
static IBox ib_refine(const IBox& b) {
    IBox r;
    for (int d = 0; d < 3; ++d) { r.lo[d] = 2 * b.lo[d]; r.hi[d] = 2 * b.hi[d] + 1; }
    return r;
}
static IBox ib_shift(const IBox& b, const int* s) {
    IBox r;
    for (int d = 0; d < 3; ++d) { r.lo[d] = b.lo[d] + s[d]; r.hi[d] = b.hi[d] + s[d]; }
    return r;
}
static long long ib_cells(const IBox& b) {
    return ib_empty(b) ? 0 : (long long)(b.hi[0] - b.lo[0] + 1) * (b.hi[1] - b.lo[1] + 1) * (b.hi[2] - b.lo[2] + 1);
}
static bool ib_same(const IBox& a, const IBox& b) {
    for (int d = 0; d < 3; ++d)
        if (a.lo[d] != b.lo[d] || a.hi[d] != b.hi[d]) return false;
    return true;
}
// a minus b as up to 6 disjoint boxes
static void ib_subtract(const IBox& a, const IBox& b, std::vector<IBox>& out) {
    IBox i;
    if (!ib_isect(a, b, i)) {
        out.push_back(a);
        return;
    }
    IBox r = a;
    for (int d = 0; d < 3; ++d) {
        if (r.lo[d] < i.lo[d]) {
            IBox p = r;
            p.hi[d] = i.lo[d] - 1;
            out.push_back(p);
            r.lo[d] = i.lo[d];
        }
        if (r.hi[d] > i.hi[d]) {
            IBox p = r;
            p.lo[d] = i.hi[d] + 1;
            out.push_back(p);
            r.hi[d] = i.hi[d];
        }
    }
}
static void list_subtract(std::vector<IBox>& list, const IBox& b) {
    std::vector<IBox> out;
    for (const IBox& a : list) ib_subtract(a, b, out);
    list.swap(out);
}

// Bucketed lookup of the boxes of one level (buckets of 16^3 cells over the domain).
struct BoxIndex {
    static constexpr int BS = 16;
    std::vector<IBox> boxes;
    IBox dom{};
    int nb[3] = {0, 0, 0};
    std::vector<std::vector<int>> bucket;
    void build(const std::vector<IBox>& bx, const IBox& d) {
        boxes = bx;
        dom = d;
        for (int e = 0; e < 3; ++e) nb[e] = (d.hi[e] - d.lo[e] + BS) / BS;
        bucket.assign((size_t)nb[0] * nb[1] * nb[2], {});
        for (int b = 0; b < (int)bx.size(); ++b) {
            IBox c;
            if (!ib_isect(bx[b], dom, c)) continue;
            int lo[3], hi[3];
            for (int e = 0; e < 3; ++e) {
                lo[e] = (c.lo[e] - dom.lo[e]) / BS;
                hi[e] = (c.hi[e] - dom.lo[e]) / BS;
            }
            for (int k = lo[2]; k <= hi[2]; ++k)
                for (int j = lo[1]; j <= hi[1]; ++j)
                    for (int i = lo[0]; i <= hi[0]; ++i) bucket[(size_t)i + nb[0] * ((size_t)j + (size_t)nb[1] * k)].push_back(b);
        }
    }
    int find(const int* c) const {
        for (int e = 0; e < 3; ++e)
            if (c[e] < dom.lo[e] || c[e] > dom.hi[e]) return -1;
        const size_t q = (size_t)((c[0] - dom.lo[0]) / BS) +
                         nb[0] * ((size_t)((c[1] - dom.lo[1]) / BS) + (size_t)nb[1] * ((c[2] - dom.lo[2]) / BS));
        for (int b : bucket[q]) {
            const IBox& B = boxes[b];
            if (c[0] >= B.lo[0] && c[0] <= B.hi[0] && c[1] >= B.lo[1] && c[1] <= B.hi[1] && c[2] >= B.lo[2] &&
                c[2] <= B.hi[2])
                return b;
        }
        return -1;
    }
    // boxes intersecting r (r clipped to the domain), ascending
    std::vector<int> query(const IBox& r) const {
        std::vector<int> out;
        IBox c;
        if (!ib_isect(r, dom, c)) return out;
        int lo[3], hi[3];
        for (int e = 0; e < 3; ++e) {
            lo[e] = (c.lo[e] - dom.lo[e]) / BS;
            hi[e] = (c.hi[e] - dom.lo[e]) / BS;
        }
        for (int k = lo[2]; k <= hi[2]; ++k)
            for (int j = lo[1]; j <= hi[1]; ++j)
                for (int i = lo[0]; i <= hi[0]; ++i)
                    for (int b : bucket[(size_t)i + nb[0] * ((size_t)j + (size_t)nb[1] * k)]) {
                        IBox t;
                        if (ib_isect(boxes[b], c, t)) out.push_back(b);
                    }
        std::sort(out.begin(), out.end());
        out.erase(std::unique(out.begin(), out.end()), out.end());
        return out;
    }
};

// ================================================================ device tags
// Cut-cell data of one box for the coarse-fine operators: kind OCFD_BOX_* and,
// for a cut box, its z-invariant flags / volume fractions over grow(bx, 5) in x, y
struct EbRef {
    const uint32_t* flag;
    const double* vf;
    int gx, x0, y0;
    int kind;
};
struct CfTag {  // fine cells interpolated from one coarse box, by parent cell
    int fbox, cbox;
    int lo[3], hi[3];    // parent cells (coarse, inside the domain)
    int flo[3], fhi[3];  // the children to fill (fine, inside the domain)
    int shift[3];        // fine cell in the fine box's index space = domain cell - shift
    EbRef ceb;           // the coarse box's cut-cell data
};
struct AvgTag {  // coarse cells averaged from one fine box
    int cbox, fbox;
    int lo[3], hi[3];
    EbRef feb;           // the fine box's cut-cell data (volume-fraction weights)
};
struct CopyTag {  // regrid: new box dst <- old box src
    int dst, src;
    int lo[3], hi[3];
};
struct RefluxCell {
    long long u, uns;  // element of component 0 in the coarse state buffer, component stride
    int first, count;  // faces
    const double* vf;  // volume fraction of a cut coarse cell (nullptr: 1)
};
struct RefluxFace {
    int d;
    double sgn;      // +1: the coarse cell is on the low side of the face
    long long c, cns;  // coarse register element (component 0), component stride
    long long f[4];    // the four fine register elements (component 0)
    long long fns;
};
struct TimeMix {
    const double* src[4];
    double a[4];
    // z faces of the coarse level whose outside ghosts are not filled
    int zvirt, zlo, zhi, zsign[2];
};
struct TagGeom {
    int dom_lo[3], dom_hi[3];
    int bs[3], nb[3];  // block size in this level's cells, blocks per direction
    int nbuf;
    double thr;
    int zvirt;         // z ghosts outside the domain unfilled: rho there equals the boundary cell's
};
struct AmrStates {
    StepState* s[OCFD_AMR_MAX_LEVELS];
    int n;
    double fixed_dt;  // > 0: the coarse step is this dt (reacting hierarchy, Source/Advance.cpp:54-57)
};

// monotonized-central slope of c between m and p: 0 unless both one-sided
// differences are non-zero with one sign, else min(|dc|, 2 min(|dl|, |dr|)) with
// the sign of dc.  The sign tests and the minima run on the integer pipes (the
// bits of non-negative doubles order as their values; dc has the sign of dl);
// only NaN differences, and a product dl dr that would underflow (|dl dr| below
// 5e-324), select differently from the floating-point tests.
__device__ __forceinline__ double mc_slope(double m, double c, double p) {
    const double dl = c - m, dr = p - c;
    const long long mag = 0x7fffffffffffffffLL;
    const long long il = __double_as_longlong(dl), ir = __double_as_longlong(dr);
    const long long al = il & mag, ar = ir & mag;
    if ((il ^ ir) < 0 || al == 0 || ar == 0) return 0.0;
    const double dc = 0.5 * (dl + dr);
    const long long adc = __double_as_longlong(dc) & mag;
    const long long a2 = __double_as_longlong(2.0 * __longlong_as_double(al < ar ? al : ar));
    const double a = __longlong_as_double(adc < a2 ? adc : a2);
    return il < 0 ? -a : a;
}

__device__ __forceinline__ double mixed(const TimeMix& m, long long q) {
    double v = 0.0;
#pragma unroll
    for (int s = 0; s < 4; ++s)
        if (m.a[s] != 0.0) v += m.a[s] * m.src[s][q];
    return v;
}

__global__ void k_cf_interp(const CfTag* __restrict__ tags, const long long* __restrict__ start,
                            const int* __restrict__ chunk, int ntag, long long total,
                            const FabGeom* __restrict__ ffabs, double* dst, const FabGeom* __restrict__ cfabs,
                            TimeMix mix, int ncomp) {
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int t = find_tag_chunked(start, chunk, ntag, idx);
        const CfTag& T = tags[t];
        int pi, pj, pk;
        region_cell(T.lo, T.hi, idx - start[t], pi, pj, pk);
        const FabGeom& cf = cfabs[T.cbox];
        const FabGeom& ff = ffabs[T.fbox];
        const long long c = fab_index(cf, pi, pj, pk);
        const long long sy = cf.g[0], sz = (long long)cf.g[0] * cf.g[1];
        const long long o = fab_index(ff, 2 * pi - T.shift[0], 2 * pj - T.shift[1], 2 * pk - T.shift[2]);
        const long long fy = ff.g[0], fz = (long long)ff.g[0] * ff.g[1];
        // children of this parent inside the region (bit ii + 2 jj + 4 kk)
        unsigned inside = 0;
#pragma unroll
        for (int q8 = 0; q8 < 8; ++q8) {
            const int ci = 2 * pi + (q8 & 1), cj = 2 * pj + ((q8 >> 1) & 1), ck = 2 * pk + (q8 >> 2);
            if (ci >= T.flo[0] && ci <= T.fhi[0] && cj >= T.flo[1] && cj <= T.fhi[1] && ck >= T.flo[2] &&
                ck <= T.fhi[2])
                inside |= 1u << q8;
        }
        // piecewise-constant interpolation where the parent or one of its face
        // neighbours is cut or covered (z neighbours share the parent's column)
        bool flat = T.ceb.kind == OCFD_BOX_COVERED;
        if (T.ceb.kind == OCFD_BOX_CUT) {
            const uint32_t* fl = T.ceb.flag + (pi - T.ceb.x0) + (long long)(pj - T.ceb.y0) * T.ceb.gx;
            flat = ((fl[0] | fl[-1] | fl[1] | fl[-T.ceb.gx] | fl[T.ceb.gx]) & 3u) != 0u;
        }
        // a z neighbour outside a z face with unfilled ghosts is the parent itself
        // (the boundary cell and the first mirror cell coincide), signs per BC
        const bool zl = mix.zvirt && pk - 1 < mix.zlo, zh = mix.zvirt && pk + 1 > mix.zhi;
        for (int n = 0; n < ncomp; ++n) {
            const long long q = c + n * cf.ns;
            const double v0 = mixed(mix, q);
            const bool flip_l = zl && n >= 1 && n <= 3 && ((mix.zsign[0] >> (n - 1)) & 1);
            const bool flip_h = zh && n >= 1 && n <= 3 && ((mix.zsign[1] >> (n - 1)) & 1);
            const double vzm = zl ? (flip_l ? -v0 : v0) : mixed(mix, q - sz);
            const double vzp = zh ? (flip_h ? -v0 : v0) : mixed(mix, q + sz);
            const double sx_ = flat ? 0.0 : mc_slope(mixed(mix, q - 1), v0, mixed(mix, q + 1));
            const double sy_ = flat ? 0.0 : mc_slope(mixed(mix, q - sy), v0, mixed(mix, q + sy));
            const double sz_ = flat ? 0.0 : mc_slope(vzm, v0, vzp);
            // child (ii, jj, kk) = v0 +- s_x / 4 +- s_y / 4 +- s_z / 4, summed in x, y, z
            // order from shared partial sums (s / 4 is exact, so each sum is the
            // same rounding as the fused multiply-add of the slope)
            const double hx = 0.25 * sx_, hy = 0.25 * sy_, hz = 0.25 * sz_;
            const double px[2] = {v0 - hx, v0 + hx};
            const double pxy[4] = {px[0] - hy, px[1] - hy, px[0] + hy, px[1] + hy};
            double* d = dst + o + n * ff.ns;
#pragma unroll
            for (int q8 = 0; q8 < 8; ++q8) {
                const int ii = q8 & 1, jj = (q8 >> 1) & 1, kk = q8 >> 2;
                if (inside & (1u << q8)) d[ii + jj * fy + kk * fz] = kk ? pxy[q8 & 3] + hz : pxy[q8 & 3] - hz;
            }
        }
    }
}

__global__ void k_avg_down(const AvgTag* __restrict__ tags, const long long* __restrict__ start, int ntag,
                           long long total, const FabGeom* __restrict__ cfabs, double* cdst,
                           const FabGeom* __restrict__ ffabs, const double* __restrict__ fsrc, int ncomp) {
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int t = find_tag<AvgTag>(start, ntag, idx);
        const AvgTag& T = tags[t];
        int i, j, k;
        region_cell(T.lo, T.hi, idx - start[t], i, j, k);
        const FabGeom& cf = cfabs[T.cbox];
        const FabGeom& ff = ffabs[T.fbox];
        const long long o = fab_index(cf, i, j, k);
        const long long f0 = fab_index(ff, 2 * i, 2 * j, 2 * k);
        const long long sy = ff.g[0], sz = (long long)ff.g[0] * ff.g[1];
        if (T.feb.kind == OCFD_BOX_REGULAR) {
            for (int n = 0; n < ncomp; ++n) {
                const double* p = fsrc + f0 + n * ff.ns;
                double s = 0.0;
                for (int kk = 0; kk < 2; ++kk)
                    for (int jj = 0; jj < 2; ++jj)
                        for (int ii = 0; ii < 2; ++ii) s += p[ii + jj * sy + kk * sz];
                cdst[o + n * cf.ns] = 0.125 * s;
            }
        } else {
            // EB_average_down (Source/EBR.cpp:549-557): fine cells weighted by
            // their volume fractions; a coarse cell whose children are all
            // covered takes its first child
            double w[8], wt = 0.0;
            for (int q8 = 0; q8 < 8; ++q8) {
                const int ii = q8 & 1, jj = (q8 >> 1) & 1;
                w[q8] = T.feb.kind == OCFD_BOX_COVERED
                            ? 0.0
                            : T.feb.vf[(2 * i + ii - T.feb.x0) + (long long)(2 * j + jj - T.feb.y0) * T.feb.gx];
                wt += w[q8];
            }
            for (int n = 0; n < ncomp; ++n) {
                const double* p = fsrc + f0 + n * ff.ns;
                double s = 0.0;
                for (int q8 = 0; q8 < 8; ++q8) {
                    const int ii = q8 & 1, jj = (q8 >> 1) & 1, kk = q8 >> 2;
                    s += w[q8] * p[ii + jj * sy + kk * sz];
                }
                cdst[o + n * cf.ns] = wt > 0.0 ? s / wt : p[0];
            }
        }
    }
}

__global__ void k_reflux(const RefluxCell* __restrict__ cells, int ncell, const RefluxFace* __restrict__ faces,
                         const double* __restrict__ creg, const double* __restrict__ freg, double* U,
                         double dxi0, double dxi1, double dxi2, int ncomp) {
    const double dxinv[3] = {dxi0, dxi1, dxi2};
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += gridDim.x * blockDim.x) {
        const RefluxCell& C = cells[c];
        const double vf = C.vf ? *C.vf : 1.0;
        if (!(vf > 0.0)) continue;
        for (int n = 0; n < ncomp; ++n) {
            double acc = 0.0;
            for (int q = C.first; q < C.first + C.count; ++q) {
                const RefluxFace& F = faces[q];
                const double fc = creg[F.c + n * F.cns];
                const double ff = 0.25 * (freg[F.f[0] + n * F.fns] + freg[F.f[1] + n * F.fns] +
                                          freg[F.f[2] + n * F.fns] + freg[F.f[3] + n * F.fns]);
                acc += F.sgn * dxinv[F.d] * (fc - ff);
            }
            U[C.u + n * C.uns] += C.vf ? acc / vf : acc;
        }
    }
}

__global__ void k_copy_tags(const CopyTag* __restrict__ tags, const long long* __restrict__ start, int ntag,
                            long long total, const FabGeom* __restrict__ dfabs, double* dst,
                            const FabGeom* __restrict__ sfabs, const double* __restrict__ src, int ncomp) {
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int t = find_tag<CopyTag>(start, ntag, idx);
        const CopyTag& T = tags[t];
        int i, j, k;
        region_cell(T.lo, T.hi, idx - start[t], i, j, k);
        const FabGeom& fd = dfabs[T.dst];
        const FabGeom& fs = sfabs[T.src];
        const long long d = fab_index(fd, i, j, k), s = fab_index(fs, i, j, k);
        for (int n = 0; n < ncomp; ++n) dst[d + n * fd.ns] = src[s + n * fs.ns];
    }
}

// tag_dengrad, Source/Tagging.H:11-36, marking the blocks of the next level that
// hold a tagged cell or one within n_error_buf cells of it
__global__ void k_tag_dengrad(const FabGeom* __restrict__ lfabs, const long long* __restrict__ cstart, int nbox,
                              long long total, const double* __restrict__ U, TagGeom g, unsigned char* blk) {
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int b = find_tag<FabGeom>(cstart, nbox, idx);
        const FabGeom& f = lfabs[b];
        int c3[3];
        region_cell(f.lo, f.hi, idx - cstart[b], c3[0], c3[1], c3[2]);
        const long long c = fab_index(f, c3[0], c3[1], c3[2]);
        const long long sy = f.g[0], sz = (long long)f.g[0] * f.g[1];
        const double r = U[c];
        const double rzp = (g.zvirt && c3[2] + 1 > g.dom_hi[2]) ? r : U[c + sz];
        const double rzm = (g.zvirt && c3[2] - 1 < g.dom_lo[2]) ? r : U[c - sz];
        double ax = fabs(U[c + 1] - r), ay = fabs(U[c + sy] - r), az = fabs(rzp - r);
        ax = fmax(ax, fabs(r - U[c - 1]));
        ay = fmax(ay, fabs(r - U[c - sy]));
        az = fmax(az, fabs(r - rzm));
        if (fmax(ax, fmax(ay, az)) >= g.thr) {
            int lo[3], hi[3];
            for (int d = 0; d < 3; ++d) {
                lo[d] = (max(c3[d] - g.nbuf, g.dom_lo[d]) - g.dom_lo[d]) / g.bs[d];
                hi[d] = (min(c3[d] + g.nbuf, g.dom_hi[d]) - g.dom_lo[d]) / g.bs[d];
            }
            for (int kb = lo[2]; kb <= hi[2]; ++kb)
                for (int jb = lo[1]; jb <= hi[1]; ++jb)
                    for (int ib = lo[0]; ib <= hi[0]; ++ib)
                        blk[ib + (long long)g.nb[0] * (jb + (long long)g.nb[1] * kb)] = 1;
        }
    }
}

__global__ void k_amr_begin(AmrStates S) {
    StepState* s0 = S.s[0];
    double est = __longlong_as_double(0x7FF0000000000000LL);
    for (int l = 0; l < S.n; ++l) {
        const double e = __longlong_as_double((long long)S.s[l]->cfl_min) * (double)(1 << l);
        est = e < est ? e : est;
    }
    double dt = s0->cfl * est;
    if (S.fixed_dt > 0) {
        dt = S.fixed_dt;
    } else {
        if (s0->dt_prev > 0 && dt > 1.1 * s0->dt_prev) dt = 1.1 * s0->dt_prev;
        if (s0->time + dt > s0->stop_time - 0.001 * dt) dt = s0->stop_time - s0->time;
        if (dt < 0) dt = 0;
    }
    for (int l = 0; l < S.n; ++l) {
        S.s[l]->dt = dt / (double)(1 << l);
        S.s[l]->time = s0->time;
        S.s[l]->cfl_min = 0x7FF0000000000000ULL;
    }
}

__global__ void k_sub_end(StepState* s) { s->time += s->dt; }

__global__ void k_amr_end(AmrStates S) {
    StepState* s0 = S.s[0];
    s0->time += s0->dt;
    s0->dt_prev = s0->dt;
    for (int l = 1; l < S.n; ++l) S.s[l]->time = s0->time;
}

__global__ void k_amr_sync(AmrStates S, double t, int reset) {
    for (int l = 0; l < S.n; ++l) {
        S.s[l]->time = t;
        S.s[l]->stop_time = S.s[0]->stop_time;
        if (reset) {
            S.s[l]->dt = 0;
            S.s[l]->dt_prev = -1.0;
        }
    }
}

__global__ void k_amr_stop(AmrStates S, double t) {
    for (int l = 0; l < S.n; ++l) S.s[l]->stop_time = t;
}

__global__ void k_copy_step(StepState* dst, const StepState* src, const StepState* est) {
    *dst = *src;
    dst->cfl_min = est ? est->cfl_min : 0x7FF0000000000000ULL;
}

__global__ void k_reset_cfl_all(AmrStates S) {
    for (int l = 0; l < S.n; ++l) S.s[l]->cfl_min = 0x7FF0000000000000ULL;
}

__global__ void k_estdt_into(const FabGeom* __restrict__ fabs, const long long* __restrict__ start, int nbox,
                             long long total, const double* __restrict__ U, DevParm P, double dx0, double dx1,
                             double dx2, unsigned long long* out) {
    const double dx[3] = {dx0, dx1, dx2};
    CflSpeeds spd;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int b = find_tag<FabGeom>(start, nbox, idx);
        const FabGeom& f = fabs[b];
        int i, j, k;
        region_cell(f.lo, f.hi, idx - start[b], i, j, k);
        const long long c = fab_index(f, i, j, k);
        double u[5];
        for (int n = 0; n < 5; ++n) u[n] = U[c + n * f.ns];
        spd.add(P, u);
    }
    block_cfl_atomic(spd, dx, out);
}

// ================================================================ hierarchy
template <class Tag>
struct DevTags {
    Tag* d = nullptr;
    long long* start = nullptr;
    int* chunk = nullptr;  // find_tag_chunked table
    int n = 0;
    long long total = 0;
    void release(DevPool* pool) {
        dev_free(d, pool);
        dev_free(start, pool);
        dev_free(chunk, pool);
        d = nullptr;
        start = nullptr;
        chunk = nullptr;
        n = 0;
        total = 0;
    }
    ocfd_status set(const std::vector<Tag>& v, DevPool* pool) {
        release(pool);
        n = (int)v.size();
        return upload_tags(v, &d, &start, &total, pool, &chunk);
    }
};

// ------------------------------------------------------- reacting hierarchy
// One stage's combination over every component of a level's cells,
// out = a U^n + b (S + dt L(S)) (the Heun / Shu-Osher forms of the flow step,
// Source/CHEM/FlowAdvance.cpp:64-88), dt the level's step.
__global__ void k_amr_combine(const FabGeom* __restrict__ fabs, const long long* __restrict__ start, int nbox,
                              long long total, double* out, const double* __restrict__ U0,
                              const double* __restrict__ S, const double* __restrict__ R, double a, double b,
                              const StepState* st, int ncomp) {
    const double dt = st->dt;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int bx = find_tag<FabGeom>(start, nbox, idx);
        const FabGeom& f = fabs[bx];
        int i, j, k;
        region_cell(f.lo, f.hi, idx - start[bx], i, j, k);
        const long long c = fab_index(f, i, j, k);
        for (int n = 0; n < ncomp; ++n) {
            const long long q = c + n * f.ns;
            out[q] = a * U0[q] + b * (S[q] + dt * R[q]);
        }
    }
}

// The flow (5) and species (9) face fluxes of one box, as its multispecies
// kernel chain left them, into the flux registers of its level: weight w dt on
// every face of a coarse box next to a finer level (flux_reg CrseAdd), on the
// box's own boundary faces of a fine box (FineAdd) - the flux_reg and
// flux_reg_spec additions of compute_dSdt_multi (Source/CHEM/FlowAdvance.cpp:
// 92-496)
struct ChemRegBox {
    View<double> flux[3], fluxs[3];
    View<double> creg[3];
    View<double> fplane[3][2];
    int bits;
    int lo[3], hi[3];
    double w;
};

__global__ void k_amr_chem_reg(ChemRegBox R, const StepState* st) {
    const double wdt = R.w * st->dt;
    const int n[3] = {R.hi[0] - R.lo[0] + 1, R.hi[1] - R.lo[1] + 1, R.hi[2] - R.lo[2] + 1};
    const long long nf[3] = {(long long)(n[0] + 1) * n[1] * n[2], (long long)n[0] * (n[1] + 1) * n[2],
                             (long long)n[0] * n[1] * (n[2] + 1)};
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < nf[0] + nf[1] + nf[2];
         idx += (long long)gridDim.x * blockDim.x) {
        const int d = idx < nf[0] ? 0 : (idx < nf[0] + nf[1] ? 1 : 2);
        const long long loc = idx - (d == 0 ? 0 : (d == 1 ? nf[0] : nf[0] + nf[1]));
        const int fx = n[0] + (d == 0), fy = n[1] + (d == 1);
        const int i = R.lo[0] + (int)(loc % fx), j = R.lo[1] + (int)((loc / fx) % fy),
                  k = R.lo[2] + (int)(loc / ((long long)fx * fy));
        const int g = d == 0 ? i : (d == 1 ? j : k);
        const bool plane = (R.bits & FLUX_ACC_PLANES) && (g == R.lo[d] || g == R.hi[d] + 1);
        if (!(R.bits & FLUX_ACC_ALL) && !plane) continue;
        double F[14];
        for (int m = 0; m < 5; ++m) F[m] = R.flux[d](i, j, k, m);
        for (int m = 0; m < NSP; ++m) F[5 + m] = R.fluxs[d](i, j, k, m);
        if (R.bits & FLUX_ACC_ALL)
            for (int m = 0; m < 14; ++m) R.creg[d](i, j, k, m) += wdt * F[m];
        if (plane) {
            const View<double>& pl = R.fplane[d][g == R.lo[d] ? 0 : 1];
            for (int m = 0; m < 14; ++m) pl(i, j, k, m) += wdt * F[m];
        }
    }
}

struct AmrLev {
    ocfd_level* L = nullptr;
    std::vector<IBox> boxes;
    IBox dom{};
    double dx[3] = {0, 0, 0};
    int bf[3] = {1, 1, 1};           // blocking factor of this level's boxes (lev >= 1)
    DevTags<CfTag> cf;               // coarse-fine ghost cells (lev >= 1)
    DevTags<AvgTag> avg;             // average-down into lev - 1
    RefluxCell* d_rc = nullptr;      // reflux of lev - 1 around this level
    RefluxFace* d_rf = nullptr;
    int nrc = 0;
    double* freg = nullptr;          // fine side of the register with lev - 1: boundary planes
    long long freg_elems = 0;
    double* creg = nullptr;          // coarse side of the register with lev + 1: face arrays
    long long creg_elems = 0;
    long long leaf = 0;
    unsigned char* d_blk = nullptr;  // tag blocks of lev + 1
    long long nblk_cap = 0;
    // reacting hierarchy: the multispecies right-hand side (FAB layout of the
    // level's state), the per-box scratch of its kernel chain, and the argument
    // blocks of every box per state buffer
    double* rhs = nullptr;
    double* cscr = nullptr;
    std::vector<ChemBoxArgs> cargs[4];
    void release_tables(DevPool* pool) {
        cf.release(pool);
        avg.release(pool);
        dev_free(d_rc, pool);
        dev_free(d_rf, pool);
        dev_free(freg, pool);
        dev_free(creg, pool);
        dev_free(rhs, pool);
        dev_free(cscr, pool);
        d_rc = nullptr;
        d_rf = nullptr;
        nrc = 0;
        freg = creg = nullptr;
        rhs = cscr = nullptr;
        for (auto& c : cargs) c.clear();
        freg_elems = creg_elems = 0;
    }
};

}  // namespace ocfd

struct ocfd_amr {
    ocfd::DevPool pool;   // destroyed last: every level and table returns its blocks here
    ocfd_context* ctx = nullptr;
    ocfd_amr_desc desc{};
    std::vector<ocfd_box> boxes0;
    int nlev = 0;
    ocfd::AmrLev lev[OCFD_AMR_MAX_LEVELS];
    bool periodic[3] = {false, false, false};
    cudaGraphExec_t graph = nullptr;
    unsigned graph_flags = ~0u;
    bool graph_ok = false;
    bool need_estdt = true;
    long long steps = 0;
    int launches = 0;          // kernels of the captured coarse step
    bool has_eb = false;       // embedded body cutting every level
    int rk_order = 3;          // time integration of every level (rk_scheme)
    ocfd_eb_desc eb{};
    // autotuned tile shape and schedule per level index (-1: not tuned)
    int tuned_tile[OCFD_AMR_MAX_LEVELS] = {-1, -1, -1, -1, -1, -1};
    int tuned_sched[OCFD_AMR_MAX_LEVELS] = {0, 0, 0, 0, 0, 0};
    long long kernel_total = 0;  // kernels launched by this hierarchy so far
    // reacting hierarchy (ocfd_amr_create_reacting): 5 + 9 components, the
    // multispecies path of every level, chemistry substeps, species reflux
    int ncomp = 5;
    bool react = false;
    ocfd_amr_react_desc rdesc{};
};

namespace ocfd {

static const int kNest = 2;  // proper nesting: coarse cells around a fine box's coarsening

// host-side phase timing of regridding, printed to stderr when OCFD_AMR_PROFILE is set
struct PhaseTimer {
    bool on = std::getenv("OCFD_AMR_PROFILE") != nullptr;
    std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
    void mark(const char* what, cudaStream_t st) {
        if (!on) return;
        cudaStreamSynchronize(st);
        const auto n = std::chrono::steady_clock::now();
        std::fprintf(stderr, "[amr] %-28s %8.3f ms\n", what, std::chrono::duration<double, std::milli>(n - t).count());
        t = n;
    }
};

static IBox level_domain(const ocfd_amr* H, int l) {
    IBox d = ib_of(H->desc.domain);
    for (int e = 0; e < 3; ++e) {
        d.lo[e] = d.lo[e] << l;
        d.hi[e] = ((d.hi[e] + 1) << l) - 1;
    }
    return d;
}

static long long fab_index_h(const FabGeom& f, int i, int j, int k) {
    return f.off + (long long)(i - f.lo[0] + NGR) + (long long)(j - f.lo[1] + NGR) * f.g[0] +
           (long long)(k - f.lo[2] + NGR) * f.g[0] * f.g[1];
}

static AmrStates states(const ocfd_amr* H) {
    AmrStates S{};
    S.n = H->nlev;
    S.fixed_dt = H->react ? H->rdesc.dt : 0.0;
    for (int l = 0; l < H->nlev; ++l) S.s[l] = H->lev[l].L->d_step;
    return S;
}

static ocfd_status ensure_d(ocfd_level* L) {
    if (L->nbuf >= 4) return OCFD_OK;
    L->buf[3] = static_cast<double*>(dev_alloc(sizeof(double) * L->elems, L->pool));
    if (!L->buf[3]) return fail(OCFD_OUT_OF_MEMORY, "AMR: fourth state buffer");
    L->nbuf = 4;
    return OCFD_OK;
}

static ocfd_status make_level(ocfd_amr* H, int l, const std::vector<IBox>& boxes, int nbuf, ocfd_level** out) {
    std::vector<ocfd_box> ob;
    for (const IBox& b : boxes) ob.push_back(ob_of(b));
    ocfd_level_desc d{};
    d.nbox = (int)ob.size();
    d.boxes = ob.data();
    d.domain = ob_of(level_domain(H, l));
    for (int e = 0; e < 3; ++e) {
        d.lo_bc[e] = H->desc.lo_bc[e];
        d.hi_bc[e] = H->desc.hi_bc[e];
        d.dx[e] = H->desc.dx[e] / (double)(1 << l);
        d.prob_lo[e] = H->desc.prob_lo[e];
    }
    d.bc_case = H->desc.bc_case;
    std::memcpy(d.case_params, H->desc.case_params, sizeof(d.case_params));
    d.tile = H->tuned_tile[l];
    ocfd_status s = level_alloc(H->ctx, &d, nbuf, out, &H->pool, H->ncomp);
    if (s == OCFD_OK) (*out)->sched = H->tuned_sched[l];
    if (s == OCFD_OK) (*out)->rk_order = H->rk_order;
    if (s == OCFD_OK && H->has_eb) s = eb_setup(*out, H->eb);
    if (s == OCFD_OK && H->has_eb) s = rebuild_fill_tags(*out);
    return s;
}

static EbRef eb_ref(const ocfd_level* L, int b) {
    EbRef r{};
    r.kind = eb_box_class(L, b);
    if (r.kind == OCFD_BOX_CUT) {
        r.vf = eb_box_vfrac(L, b, &r.gx);
        r.flag = eb_box_flag(L, b);
        r.x0 = L->boxes[b].lo[0] - EB_GEOM_GROW;
        r.y0 = L->boxes[b].lo[1] - EB_GEOM_GROW;
    }
    return r;
}

// periodic images (shift vectors) of a region that meet the domain
static void periodic_shifts(const ocfd_amr* H, const IBox& dom, std::vector<std::array<int, 3>>& out) {
    out.clear();
    int period[3];
    for (int e = 0; e < 3; ++e) period[e] = dom.hi[e] - dom.lo[e] + 1;
    for (int sx = -1; sx <= 1; ++sx)
        for (int sy = -1; sy <= 1; ++sy)
            for (int sz = -1; sz <= 1; ++sz) {
                const int s[3] = {sx, sy, sz};
                bool ok = true;
                for (int e = 0; e < 3; ++e)
                    if (s[e] != 0 && !H->periodic[e]) ok = false;
                if (ok) out.push_back({sx * period[0], sy * period[1], sz * period[2]});
            }
}

// Fine cells of `regions` (per fine box) that take their value from level f-1:
// split by the coarse box holding their parent, periodic images resolved.
static ocfd_status build_cf_tags(const ocfd_amr* H, int f, const std::vector<std::vector<IBox>>& regions,
                                 std::vector<CfTag>& out) {
    const AmrLev& C = H->lev[f - 1];
    const IBox fdom = level_domain(H, f);
    BoxIndex cidx;
    cidx.build(C.boxes, C.dom);
    std::vector<std::array<int, 3>> shifts;
    periodic_shifts(H, fdom, shifts);
    for (int b = 0; b < (int)regions.size(); ++b) {
        for (const IBox& P : regions[b]) {
            long long need = ib_cells(P), got = 0;
            for (const auto& sh : shifts) {
                // cells g of P with g + sh inside the domain
                IBox Qs;
                if (!ib_isect(ib_shift(P, sh.data()), fdom, Qs)) continue;
                const IBox Qc = ib_coarsen(Qs);
                for (int cb : cidx.query(Qc)) {
                    IBox I;
                    if (!ib_isect(Qc, C.boxes[cb], I)) continue;
                    IBox Fr;
                    if (!ib_isect(ib_refine(I), Qs, Fr)) continue;
                    const IBox Pc = ib_coarsen(Fr);
                    CfTag t{};
                    t.fbox = b;
                    t.cbox = cb;
                    t.ceb = eb_ref(C.L, cb);
                    for (int e = 0; e < 3; ++e) {
                        t.lo[e] = Pc.lo[e];
                        t.hi[e] = Pc.hi[e];
                        t.flo[e] = Fr.lo[e];
                        t.fhi[e] = Fr.hi[e];
                        t.shift[e] = sh[e];
                    }
                    out.push_back(t);
                    got += ib_cells(Fr);
                }
            }
            if (got != need) return fail(OCFD_BAD_ARG, "AMR: a fine level is not properly nested in the level below");
        }
    }
    return OCFD_OK;
}

// in-domain ghost cells of each fine box not covered by the level's valid boxes
static void ghost_regions(const ocfd_amr* H, int f, std::vector<std::vector<IBox>>& regions) {
    const AmrLev& F = H->lev[f];
    const IBox fdom = level_domain(H, f);
    std::vector<std::array<int, 3>> shifts;
    periodic_shifts(H, fdom, shifts);
    regions.assign(F.boxes.size(), {});
    for (size_t b = 0; b < F.boxes.size(); ++b) {
        IBox R = ib_grow(F.boxes[b], box_nfill(F.L, (int)b));
        for (int e = 0; e < 3; ++e)
            if (!H->periodic[e]) {
                R.lo[e] = std::max(R.lo[e], fdom.lo[e]);
                R.hi[e] = std::min(R.hi[e], fdom.hi[e]);
            }
        std::vector<IBox> list{R};
        for (const auto& sh : shifts)
            for (const IBox& Q : F.boxes) {
                IBox t;
                const IBox Qs = ib_shift(Q, sh.data());
                if (ib_isect(R, Qs, t)) list_subtract(list, Qs);
            }
        regions[b] = list;
    }
}

static long long region_offset_plane(const IBox& pl, int i, int j, int k) {
    const long long ex = pl.hi[0] - pl.lo[0] + 1, ey = pl.hi[1] - pl.lo[1] + 1;
    return (long long)(i - pl.lo[0]) + (long long)(j - pl.lo[1]) * ex + (long long)(k - pl.lo[2]) * ex * ey;
}

// Host side of the tables between level c = f-1 and level f (ghost
// interpolation, average-down, reflux cells, the flux register layout): reads
// the hierarchy only, so the pairs of a hierarchy are built concurrently.
struct PairTables {
    ocfd_status status = OCFD_OK;
    std::vector<CfTag> cf_tags;
    std::vector<AvgTag> avg_tags;
    long long covered = 0;
    std::vector<long long> plane_off;
    std::vector<IBox> plane_box;
    long long fe = 0;
    std::vector<long long> creg_off;
    long long ce = 0;
    std::vector<RefluxCell> rc_h;
    std::vector<RefluxFace> rf_h;
};

static ocfd_status compute_pair(const ocfd_amr* H, int f, PairTables& T) {
    const AmrLev& C = H->lev[f - 1];
    const AmrLev& F = H->lev[f];
    ocfd_status s;
    {
        std::vector<std::vector<IBox>> regions;
        ghost_regions(H, f, regions);
        s = build_cf_tags(H, f, regions, T.cf_tags);
        if (s != OCFD_OK) return s;
    }
    BoxIndex cidx;
    cidx.build(C.boxes, C.dom);
    std::vector<IBox> fcoarse;
    for (const IBox& b : F.boxes) fcoarse.push_back(ib_coarsen(b));
    BoxIndex fcidx;
    fcidx.build(fcoarse, C.dom);
    {
        std::vector<AvgTag>& tags = T.avg_tags;
        long long covered = 0;
        for (int fb = 0; fb < (int)F.boxes.size(); ++fb)
            for (int cb : cidx.query(fcoarse[fb])) {
                IBox I;
                if (!ib_isect(fcoarse[fb], C.boxes[cb], I)) continue;
                AvgTag t{};
                t.cbox = cb;
                t.fbox = fb;
                t.feb = eb_ref(F.L, fb);
                for (int e = 0; e < 3; ++e) { t.lo[e] = I.lo[e]; t.hi[e] = I.hi[e]; }
                tags.push_back(t);
                covered += ib_cells(I);
            }
        T.covered = covered;
    }
    // ---- flux register layout: fine planes of every fine box
    const int nfb = (int)F.boxes.size(), ncb = (int)C.boxes.size();
    std::vector<long long>& plane_off = T.plane_off;
    std::vector<IBox>& plane_box = T.plane_box;
    plane_off.assign((size_t)nfb * 6, 0);
    plane_box.assign((size_t)nfb * 6, IBox{});
    long long fe = 0;
    for (int fb = 0; fb < nfb; ++fb)
        for (int d = 0; d < 3; ++d)
            for (int sd = 0; sd < 2; ++sd) {
                IBox pl = F.boxes[fb];
                pl.lo[d] = pl.hi[d] = (sd == 0) ? F.boxes[fb].lo[d] : F.boxes[fb].hi[d] + 1;
                plane_off[fb * 6 + 2 * d + sd] = fe;
                plane_box[fb * 6 + 2 * d + sd] = pl;
                fe += ib_cells(pl) * H->ncomp;
            }
    // ---- reflux faces grouped by uncovered coarse cell.  The coarse cells just
    // outside each fine box (one plane per side, periodic planes wrapped into
    // the domain) minus the coarsened fine boxes: rectangles, not cells, are
    // tested for cover.  A coarse cell gathers its faces in discovery order
    // (fine box, direction, side), the summation order of its reflux; the
    // cells themselves are independent, so they are kept in first-discovery
    // order.
    struct Face {
        int d, side, cb, fb;
        int cf[3];  // coarse face index
        int c[3];   // unwrapped coarse cell (transverse coordinates pick the fine faces)
    };
    std::vector<Face> faces;
    std::vector<long long> face_u;
    const IBox& cd = C.dom;
    for (int fb = 0; fb < nfb; ++fb) {
        const IBox& Fc = fcoarse[fb];
        for (int d = 0; d < 3; ++d)
            for (int sd = 0; sd < 2; ++sd) {
                IBox pl = Fc;
                pl.lo[d] = pl.hi[d] = (sd == 0) ? Fc.lo[d] - 1 : Fc.hi[d] + 1;
                const int per = cd.hi[d] - cd.lo[d] + 1;
                IBox wp = pl;  // the plane in the domain (transverse extents lie in Fc, inside it)
                if (pl.lo[d] < cd.lo[d] || pl.lo[d] > cd.hi[d]) {
                    if (!H->periodic[d]) continue;  // physical boundary
                    wp.lo[d] = wp.hi[d] = cd.lo[d] + (((pl.lo[d] - cd.lo[d]) % per) + per) % per;
                }
                std::vector<IBox> open{wp};
                for (int ob : fcidx.query(wp)) list_subtract(open, fcoarse[ob]);
                for (const IBox& r : open)
                    for (int k = r.lo[2]; k <= r.hi[2]; ++k)
                        for (int j = r.lo[1]; j <= r.hi[1]; ++j)
                            for (int i = r.lo[0]; i <= r.hi[0]; ++i) {
                                int w[3] = {i, j, k};
                                const int cb = cidx.find(w);
                                if (cb < 0) return fail(OCFD_BAD_ARG, "AMR: reflux cell outside the coarse level");
                                Face fc{};
                                fc.d = d;
                                fc.side = sd;
                                fc.cb = cb;
                                fc.fb = fb;
                                for (int e = 0; e < 3; ++e) { fc.cf[e] = w[e]; fc.c[e] = w[e]; }
                                fc.c[d] = pl.lo[d];
                                if (sd == 0) fc.cf[d] = w[d] + 1;
                                faces.push_back(fc);
                                face_u.push_back(fab_index_h(C.L->fabs[cb], w[0], w[1], w[2]));
                            }
            }
    }
    // group the faces by coarse cell (an element index of the level's state is
    // unique across its boxes) with discovery order kept inside a group: one
    // radix sort of 64-bit keys (element index, discovery index), all distinct
    if (faces.size() >= (size_t(1) << 22)) return fail(OCFD_BAD_ARG, "AMR: too many reflux faces");
    std::vector<uint64_t> key(faces.size());
    for (size_t q = 0; q < faces.size(); ++q) key[q] = ((uint64_t)face_u[q] << 22) | (uint64_t)q;
    radix_sort_u64(key);
    std::vector<int> order(faces.size()), gstart;
    for (size_t q = 0; q < key.size(); ++q) {
        order[q] = (int)(key[q] & ((1u << 22) - 1));
        if (q == 0 || (key[q] >> 22) != (key[q - 1] >> 22)) gstart.push_back((int)q);
    }
    const int ngroup = (int)gstart.size();
    gstart.push_back((int)faces.size());
    // coarse register: face arrays of the coarse boxes that own a reflux cell,
    // in box order
    std::vector<long long>& creg_off = T.creg_off;
    creg_off.assign((size_t)ncb, -1);
    long long ce = 0;
    {
        std::vector<char> owns((size_t)ncb, 0);
        for (const Face& fc : faces) owns[fc.cb] = 1;
        long long ce0 = 0;
        for (int cb = 0; cb < ncb; ++cb) {
            if (!owns[cb]) continue;
            creg_off[cb] = ce0;
            const IBox& B = C.boxes[cb];
            for (int d = 0; d < 3; ++d) {
                IBox fa = B;
                fa.hi[d] += 1;
                ce0 += ib_cells(fa) * H->ncomp;
            }
        }
        ce = ce0;
    }
    auto creg_face = [&](int cb, int d, const int* fc, long long* cns) {
        const IBox& B = C.boxes[cb];
        long long off = creg_off[cb];
        for (int e = 0; e < d; ++e) {
            IBox fa = B;
            fa.hi[e] += 1;
            off += ib_cells(fa) * H->ncomp;
        }
        IBox fa = B;
        fa.hi[d] += 1;
        *cns = ib_cells(fa);
        return off + region_offset_plane(fa, fc[0], fc[1], fc[2]);
    };
    std::vector<RefluxCell>& rc_h = T.rc_h;
    std::vector<RefluxFace>& rf_h = T.rf_h;
    rc_h.reserve(ngroup);
    rf_h.reserve(faces.size());
    for (int g = 0; g < ngroup; ++g) {
        const int q0 = gstart[g], q1 = gstart[(size_t)g + 1];
        const Face& f0 = faces[order[q0]];
        const EbRef ceb = eb_ref(C.L, f0.cb);
        if (ceb.kind == OCFD_BOX_COVERED) continue;  // covered coarse cells take no reflux
        RefluxCell cell{};
        cell.u = face_u[order[q0]];
        cell.uns = C.L->fabs[f0.cb].ns;
        if (ceb.kind == OCFD_BOX_CUT) {
            int w[3] = {f0.cf[0], f0.cf[1], f0.cf[2]};
            if (f0.side == 0) w[f0.d] -= 1;
            cell.vf = ceb.vf + (w[0] - ceb.x0) + (long long)(w[1] - ceb.y0) * ceb.gx;
        }
        cell.first = (int)rf_h.size();
        cell.count = q1 - q0;
        for (int qi = q0; qi < q1; ++qi) {
            const Face& fc = faces[order[qi]];
            RefluxFace q{};
            q.d = fc.d;
            q.sgn = fc.side == 0 ? 1.0 : -1.0;
            q.c = creg_face(fc.cb, fc.d, fc.cf, &q.cns);
            const int pidx = fc.fb * 6 + 2 * fc.d + fc.side;
            const IBox& pl = plane_box[pidx];
            q.fns = ib_cells(pl);
            const int t1 = fc.d == 0 ? 1 : 0, t2 = fc.d == 2 ? 1 : 2;
            int m = 0;
            for (int b2 = 0; b2 < 2; ++b2)
                for (int b1 = 0; b1 < 2; ++b1) {
                    int gg[3];
                    gg[fc.d] = pl.lo[fc.d];
                    gg[t1] = 2 * fc.c[t1] + b1;
                    gg[t2] = 2 * fc.c[t2] + b2;
                    q.f[m++] = plane_off[pidx] + region_offset_plane(pl, gg[0], gg[1], gg[2]);
                }
            rf_h.push_back(q);
        }
        rc_h.push_back(cell);
    }
    T.fe = fe;
    T.ce = ce;
    return OCFD_OK;
}

// Device side of a pair's tables: uploads, flux registers, the stage roles'
// register views.  Serial (the device pool is not shared between threads).
static ocfd_status apply_pair(ocfd_amr* H, int f, PairTables& T, StageRoles& rc, StageRoles& rf) {
    AmrLev& C = H->lev[f - 1];
    AmrLev& F = H->lev[f];
    const int nfb = (int)F.boxes.size(), ncb = (int)C.boxes.size();
    const std::vector<long long>& plane_off = T.plane_off;
    const std::vector<IBox>& plane_box = T.plane_box;
    const std::vector<long long>& creg_off = T.creg_off;
    const long long fe = T.fe, ce = T.ce;
    ocfd_status s = F.cf.set(T.cf_tags, &H->pool);
    if (s == OCFD_OK) s = F.avg.set(T.avg_tags, &H->pool);
    if (s != OCFD_OK) return s;
    C.leaf = C.L->ncells - T.covered;
    F.nrc = (int)T.rc_h.size();
    s = upload(&F.d_rc, T.rc_h, &H->pool);
    if (s == OCFD_OK) s = upload(&F.d_rf, T.rf_h, &H->pool);
    if (s != OCFD_OK) return s;
    F.freg_elems = fe;
    C.creg_elems = ce;
    F.freg = static_cast<double*>(dev_alloc(sizeof(double) * std::max<long long>(1, fe), &H->pool));
    C.creg = static_cast<double*>(dev_alloc(sizeof(double) * std::max<long long>(1, ce), &H->pool));
    if (!F.freg || !C.creg) return fail(OCFD_OUT_OF_MEMORY, "AMR: flux registers");
    // stage roles: register views
    rf.flux_bits.resize(nfb, 0);
    rf.fplane.resize((size_t)nfb * 6);
    for (int fb = 0; fb < nfb; ++fb) {
        rf.flux_bits[fb] |= FLUX_ACC_PLANES;
        for (int q = 0; q < 6; ++q) {
            const IBox& pl = plane_box[fb * 6 + q];
            const long long ex = pl.hi[0] - pl.lo[0] + 1, ey = pl.hi[1] - pl.lo[1] + 1;
            rf.fplane[fb * 6 + q] = View<double>{F.freg + plane_off[fb * 6 + q], ex, ex * ey, ib_cells(pl),
                                                 pl.lo[0], pl.lo[1], pl.lo[2]};
        }
    }
    rc.flux_bits.resize(ncb, 0);
    rc.creg.resize((size_t)ncb * 3);
    for (int cb = 0; cb < ncb; ++cb) {
        if (creg_off[cb] < 0) continue;
        rc.flux_bits[cb] |= FLUX_ACC_ALL;
        long long off = creg_off[cb];
        for (int d = 0; d < 3; ++d) {
            IBox fa = C.boxes[cb];
            fa.hi[d] += 1;
            const long long ex = fa.hi[0] - fa.lo[0] + 1, ey = fa.hi[1] - fa.lo[1] + 1;
            rc.creg[cb * 3 + d] = View<double>{C.creg + off, ex, ex * ey, ib_cells(fa), fa.lo[0], fa.lo[1], fa.lo[2]};
            off += ib_cells(fa) * H->ncomp;
        }
    }
    return OCFD_OK;
}

static bool fused_cfl(const ocfd_amr* H, int l) { return l == H->nlev - 1 && !H->has_eb; }

// Array4 view of components comp0 .. comp0 + ncomp - 1 of box b's FAB in `base`
static ocfd_array4 fab_view_c(const ocfd_level* L, double* base, int b, int comp0, int ncomp) {
    const FabGeom& f = L->fabs[b];
    ocfd_array4 a{};
    a.p = base + f.off + comp0 * f.ns;
    a.jstride = f.g[0];
    a.kstride = (long long)f.g[0] * f.g[1];
    a.nstride = f.ns;
    for (int d = 0; d < 3; ++d) {
        a.begin[d] = f.lo[d] - NGR;
        a.end[d] = f.hi[d] + NGR + 1;
    }
    a.ncomp = ncomp;
    return a;
}

// Reacting hierarchy: the right-hand-side buffer of level l, one scratch for its
// boxes' multispecies kernel chains (the boxes run one after the other on the
// stream, so the largest box sizes it), and every box's argument block per
// state buffer
static ocfd_status build_chem_level(ocfd_amr* H, int l) {
    AmrLev& A = H->lev[l];
    ocfd_level* L = A.L;
    dev_free(A.rhs, &H->pool);
    dev_free(A.cscr, &H->pool);
    A.rhs = static_cast<double*>(dev_alloc(sizeof(double) * L->elems, &H->pool));
    size_t need = 1;
    for (const ocfd_box& b : L->boxes) need = std::max(need, chem_rhs_scratch_doubles(b));
    A.cscr = static_cast<double*>(dev_alloc(sizeof(double) * need, &H->pool));
    if (!A.rhs || !A.cscr) return fail(OCFD_OUT_OF_MEMORY, "reacting hierarchy: right-hand-side buffers");
    const double dxinv[3] = {1.0 / L->desc.dx[0], 1.0 / L->desc.dx[1], 1.0 / L->desc.dx[2]};
    const bool visc = (H->rdesc.flags & OCFD_VISC) != 0;
    for (int i = 0; i < 4; ++i) {
        A.cargs[i].clear();
        if (i >= L->nbuf) continue;
        for (int b = 0; b < (int)L->boxes.size(); ++b) {
            ocfd_array4 S = fab_view_c(L, L->buf[i], b, 0, 5), sp = fab_view_c(L, L->buf[i], b, 5, NSP);
            ocfd_array4 d = fab_view_c(L, A.rhs, b, 0, 5), ds = fab_view_c(L, A.rhs, b, 5, NSP);
            ChemBoxArgs X{};
            chem_rhs_args(X, view_of<const double>(&S), view_of<const double>(&sp), view_of<double>(&d),
                          view_of<double>(&ds), L->boxes[b], dxinv, visc, A.cscr);
            A.cargs[i].push_back(X);
        }
    }
    return OCFD_OK;
}

static ocfd_status rebuild_tables(ocfd_amr* H) {
    // blocks of the old tables go back to the pool: nothing may still read them
    if (cudaDeviceSynchronize() != cudaSuccess) return check_launch("AMR table rebuild");
    std::vector<StageRoles> roles(H->nlev);
    for (int l = 0; l < H->nlev; ++l) {
        H->lev[l].release_tables(&H->pool);
        H->lev[l].leaf = H->lev[l].L->ncells;
        // the finest level's final state is its last substep's stage output (no
        // reflux or average-down follows), so its CFL estimate for the next step
        // is fused into that stage; coarser levels and cut levels are estimated
        // by a pass over their state at the end of the step
        roles[l].cfl = fused_cfl(H, l);
        roles[l].out3 = (l < H->nlev - 1) ? 3 : 0;
        if (l < H->nlev - 1) {
            ocfd_status s = ensure_d(H->lev[l].L);
            if (s != OCFD_OK) return s;
        }
    }
    PhaseTimer pt;
    {
        // host tables of every level pair at once, then their uploads in order
        std::vector<PairTables> T(H->nlev);
        std::vector<std::thread> workers;
        for (int f = 1; f < H->nlev; ++f)
            workers.emplace_back([H, f, &T] { T[f].status = compute_pair(H, f, T[f]); });
        for (std::thread& w : workers) w.join();
        pt.mark("    pair tables (host)", 0);
        for (int f = 1; f < H->nlev; ++f) {
            ocfd_status s = T[f].status;
            if (s == OCFD_OK) s = apply_pair(H, f, T[f], roles[f - 1], roles[f]);
            if (s != OCFD_OK) return s;
        }
        pt.mark("    pair tables (device)", 0);
    }
    for (int l = 0; l < H->nlev; ++l) {
        StageRoles& r = roles[l];
        const int nb = (int)H->lev[l].boxes.size();
        if (!r.flux_bits.empty()) {
            r.flux_bits.resize(nb, 0);
            r.creg.resize((size_t)nb * 3);
            r.fplane.resize((size_t)nb * 6);
        }
        ocfd_status s = build_stage_tables(H->lev[l].L, r);
        if (s == OCFD_OK && H->react) s = build_chem_level(H, l);
        if (s != OCFD_OK) return s;
    }
    pt.mark("    stage tables", 0);
    H->graph_ok = false;
    return OCFD_OK;
}

// ---------------------------------------------------------------- launches
static int launches_counter = 0;

static void mix_coefs(int kind, double theta, double r, double* a) {
    // kind 0..2: fine stage 1..3 of the substep starting at theta; kind 3: end (theta + r)
    double w1, w2, w3;
    auto P = [&](double th) {
        w1 = th - 5.0 / 6.0 * th * th;
        w2 = th * th / 6.0;
        w3 = 2.0 / 3.0 * th * th;
    };
    if (kind == 3) {
        P(theta + r);
    } else {
        P(theta);
        const double d1 = 1.0 - 5.0 / 3.0 * theta, d2 = theta / 3.0, d3 = 4.0 / 3.0 * theta;  // P' dt
        const double e1 = -5.0 / 3.0, e2 = 1.0 / 3.0, e3 = 4.0 / 3.0;                         // P'' dt^2
        if (kind == 1) {
            w1 += r * d1;
            w2 += r * d2;
            w3 += r * d3;
        } else if (kind == 2) {
            w1 += 0.5 * r * d1 + 0.25 * r * r * e1;
            w2 += 0.5 * r * d2 + 0.25 * r * r * e2;
            w3 += 0.5 * r * d3 + 0.25 * r * r * e3;
        }
    }
    a[0] = 1.0 - w1 - 3.0 * w2 - 0.5 * w3;
    a[1] = w1 - w2;
    a[2] = 4.0 * w2 - w3;
    a[3] = 1.5 * w3;
}

// Coarse-level weights of (A, B, C, D) for the ghosts of fine stage k of the
// substep starting at theta (k = 3: the coarse end state's ghosts, theta + r).
// SSP-RK3: the dense output of the coarse stages (mix_coefs).  Heun and Euler:
// AMReX FillPatch's linear interpolation between the coarse old (A) and new (D)
// states at the stage's time (Source/Advance.cpp:119,126; the two-level
// FillPatch of AmrLevel).
static void cf_coefs(int order, int k, double theta, double r, double* a) {
    if (order == 3) {
        mix_coefs(k, theta, r, a);
        return;
    }
    const double th = k == 3 ? theta + r : theta + r * rk_scheme(order).tfrac[k];
    a[0] = 1.0 - th;
    a[1] = 0.0;
    a[2] = 0.0;
    a[3] = th;
}

static ocfd_status launch_cf(ocfd_amr* H, int f, double* dst, const double* a, cudaStream_t st) {
    AmrLev& F = H->lev[f];
    AmrLev& C = H->lev[f - 1];
    if (F.cf.total == 0) return OCFD_OK;
    TimeMix m{};
    for (int q = 0; q < 4; ++q) {
        m.a[q] = a[q];
        m.src[q] = (a[q] != 0.0) ? C.L->buf[q] : nullptr;
        if (a[q] != 0.0 && q >= C.L->nbuf) return fail(OCFD_BAD_ARG, "AMR: time interpolation needs a missing buffer");
    }
    m.zvirt = C.L->zvirt ? 1 : 0;
    m.zlo = C.dom.lo[2];
    m.zhi = C.dom.hi[2];
    m.zsign[0] = C.L->zsign[0];
    m.zsign[1] = C.L->zsign[1];
    k_cf_interp<<<grid_for(F.cf.total, 128, H->ctx->num_sms), 128, 0, st>>>(
        F.cf.d, F.cf.start, F.cf.chunk, F.cf.n, F.cf.total, F.L->d_fabs, dst, C.L->d_fabs, m, F.L->ncomp);
    ++launches_counter;
    return check_launch("AMR coarse-fine interpolation");
}

static ocfd_status fill_level(ocfd_amr* H, int l, double* U, const double* a, double tfrac, cudaStream_t st) {
    ocfd_status s = OCFD_OK;
    if (l > 0) s = launch_cf(H, l, U, a, st);
    if (s == OCFD_OK) s = fill_exchange(H->lev[l].L, U, st);
    if (s == OCFD_OK) s = fill_physbc(H->lev[l].L, U, tfrac, st);
    ocfd_level* L = H->lev[l].L;
    launches_counter += (L->ex_total > 0) + (L->bc_total[0] > 0) + (L->bc_total[1] > 0) + (L->bc_total[2] > 0);
    return s;
}

static ocfd_status launch_avg(ocfd_amr* H, int f, const double* fsrc, double* cdst, cudaStream_t st) {
    AmrLev& F = H->lev[f];
    AmrLev& C = H->lev[f - 1];
    if (F.avg.total == 0) return OCFD_OK;
    k_avg_down<<<grid_for(F.avg.total, 256, H->ctx->num_sms), 256, 0, st>>>(
        F.avg.d, F.avg.start, F.avg.n, F.avg.total, C.L->d_fabs, cdst, F.L->d_fabs, fsrc, F.L->ncomp);
    ++launches_counter;
    return check_launch("AMR average-down");
}

// chemistry of level l over half its step, in place on U: iter_l substeps of the
// implicit cell update (Source/Advance.cpp:158-173); `renorm`: the last substep
// also renormalises the species (the finest level, whose post_timestep has no
// reflux)
static ocfd_status chem_level(ocfd_amr* H, int l, double* U, bool renorm, cudaStream_t st) {
    ocfd_level* L = H->lev[l].L;
    const int iter = l <= 2 ? std::max(1, H->rdesc.chem_substeps >> l) : 1;
    const double dt2 = 0.5 * (H->rdesc.dt / (double)(1 << l)) / iter;
    for (int s = 0; s < iter; ++s)
        for (int b = 0; b < (int)L->boxes.size(); ++b) {
            ocfd_array4 S = fab_view_c(L, U, b, 0, 5), sp = fab_view_c(L, U, b, 5, NSP);
            CellBox cb{};
            for (int d = 0; d < 3; ++d) {
                cb.lo[d] = L->boxes[b].lo[d];
                cb.n[d] = L->boxes[b].hi[d] - L->boxes[b].lo[d] + 1;
            }
            ocfd_status r = launch_chem_advance(view_of<double>(&S), view_of<double>(&sp), cb, dt2, H->ctx->parm, st,
                                                renorm && s == iter - 1);
            if (r != OCFD_OK) return r;
            ++launches_counter;
        }
    return OCFD_OK;
}

// species renormalisation of level l's state U (EBR::post_timestep, Source/EBR.cpp:333-357)
static ocfd_status renorm_level(ocfd_amr* H, int l, double* U, cudaStream_t st) {
    ocfd_level* L = H->lev[l].L;
    for (int b = 0; b < (int)L->boxes.size(); ++b) {
        ocfd_array4 S = fab_view_c(L, U, b, 0, 5), sp = fab_view_c(L, U, b, 5, NSP);
        CellBox cb{};
        for (int d = 0; d < 3; ++d) {
            cb.lo[d] = L->boxes[b].lo[d];
            cb.n[d] = L->boxes[b].hi[d] - L->boxes[b].lo[d] + 1;
        }
        ocfd_status r = launch_spec_renorm(view_of<const double>(&S), view_of<double>(&sp), cb, H->ctx->num_sms, st);
        if (r != OCFD_OK) return r;
        ++launches_counter;
    }
    return OCFD_OK;
}

// One substep of a reacting level (EBR::advance with CHEM, then post_timestep):
// chemistry over dt_l / 2, the multispecies flow step with its flux registers,
// chemistry over dt_l / 2; with a finer level: its two substeps, reflux of flow
// and species, renormalisation, average-down.
static ocfd_status advance_level_react(ocfd_amr* H, int l, int it, unsigned flags, cudaStream_t st) {
    AmrLev& A = H->lev[l];
    ocfd_level* L = A.L;
    const bool has_child = l < H->nlev - 1;
    const double theta = 0.5 * (it - 1), r = 0.5;
    const RkScheme& R = rk_scheme(H->rk_order);
    const StageRoles roles = L->roles ? *L->roles : StageRoles{};
    const int sms = H->ctx->num_sms;
    ocfd_status s = chem_level(H, l, L->buf[0], false, st);
    if (s != OCFD_OK) return s;
    if (has_child) {
        cudaMemsetAsync(A.creg, 0, sizeof(double) * std::max<long long>(1, A.creg_elems), st);
        cudaMemsetAsync(H->lev[l + 1].freg, 0, sizeof(double) * std::max<long long>(1, H->lev[l + 1].freg_elems), st);
    }
    for (int k = 0; k < R.nst && s == OCFD_OK; ++k) {
        double a[4];
        cf_coefs(R.order, k, theta, r, a);
        s = fill_level(H, l, L->buf[R.src[k]], a, R.tfrac[k], st);
        for (int b = 0; b < (int)L->boxes.size() && s == OCFD_OK; ++b) {
            ChemBoxArgs X = A.cargs[R.src[k]][b];
            X.f32 = (flags & OCFD_FLUX_FP32) ? 1 : 0;
            s = launch_chem_rhs(X, H->ctx->parm, sms, st);
            launches_counter += X.visc ? 6 : 5;
            const int bits = roles.flux_bits.empty() ? 0 : roles.flux_bits[b];
            if (s == OCFD_OK && bits) {
                ChemRegBox G{};
                for (int d = 0; d < 3; ++d) {
                    G.flux[d] = X.flux[d];
                    G.fluxs[d] = X.fluxs[d];
                    if (bits & FLUX_ACC_ALL) G.creg[d] = roles.creg[3 * b + d];
                    if (bits & FLUX_ACC_PLANES)
                        for (int sd = 0; sd < 2; ++sd) G.fplane[d][sd] = roles.fplane[6 * b + 2 * d + sd];
                    G.lo[d] = L->boxes[b].lo[d];
                    G.hi[d] = L->boxes[b].hi[d];
                }
                G.bits = bits;
                G.w = R.w[k];
                const ocfd_box& B = L->boxes[b];
                const long long nfc = 3LL * (B.hi[0] - B.lo[0] + 2) * (B.hi[1] - B.lo[1] + 2) * (B.hi[2] - B.lo[2] + 2);
                k_amr_chem_reg<<<grid_for(nfc, 256, sms), 256, 0, st>>>(G, L->d_step);
                ++launches_counter;
                s = check_launch("reacting hierarchy: flux registers");
            }
        }
        if (s != OCFD_OK) break;
        const int out = R.out[k] == RK_OUT ? roles.out3 : R.out[k];
        k_amr_combine<<<grid_for(L->ncells, 256, sms), 256, 0, st>>>(L->d_fabs, L->d_cell_start, (int)L->boxes.size(),
                                                                   L->ncells, L->buf[out], L->buf[0], L->buf[R.src[k]],
                                                                   A.rhs, R.a[k], R.b[k], L->d_step, L->ncomp);
        ++launches_counter;
        s = check_launch("reacting hierarchy: stage");
    }
    if (s != OCFD_OK) return s;
    const int fin = has_child ? 3 : 0;
    if (R.copy_out && cudaMemcpyAsync(L->buf[fin], L->buf[1], sizeof(double) * L->elems, cudaMemcpyDeviceToDevice,
                                      st) != cudaSuccess)
        return check_launch("reacting hierarchy: stage output copy");
    s = chem_level(H, l, L->buf[fin], !has_child, st);
    if (s != OCFD_OK) return s;
    if (has_child) {
        double a[4];
        cf_coefs(R.order, 3, theta, r, a);
        s = fill_level(H, l, L->buf[3], a, 1.0, st);
        for (int i = 1; i <= 2 && s == OCFD_OK; ++i) s = advance_level_react(H, l + 1, i, flags, st);
        if (s != OCFD_OK) return s;
        AmrLev& F = H->lev[l + 1];
        if (F.nrc > 0) {
            k_reflux<<<(F.nrc + 127) / 128, 128, 0, st>>>(F.d_rc, F.nrc, F.d_rf, A.creg, F.freg, L->buf[3],
                                                         1.0 / A.dx[0], 1.0 / A.dx[1], 1.0 / A.dx[2], L->ncomp);
            ++launches_counter;
        }
        s = renorm_level(H, l, L->buf[3], st);
        if (s == OCFD_OK) s = launch_avg(H, l + 1, F.L->buf[0], L->buf[3], st);
        if (s != OCFD_OK) return s;
        if (cudaMemcpyAsync(L->buf[0], L->buf[3], sizeof(double) * L->elems, cudaMemcpyDeviceToDevice, st) !=
            cudaSuccess)
            return check_launch("reacting hierarchy: D -> A");
    }
    if (l > 0) {
        k_sub_end<<<1, 1, 0, st>>>(L->d_step);
        ++launches_counter;
    }
    return check_launch("reacting hierarchy: level advance");
}

static ocfd_status advance_level(ocfd_amr* H, int l, int it, unsigned flags, cudaStream_t st) {
    if (H->react) return advance_level_react(H, l, it, flags, st);
    AmrLev& A = H->lev[l];
    ocfd_level* L = A.L;
    const bool has_child = l < H->nlev - 1;
    const double theta = 0.5 * (it - 1), r = 0.5;
    const RkScheme& R = rk_scheme(H->rk_order);
    ocfd_status s = OCFD_OK;
    if (has_child) {
        cudaMemsetAsync(A.creg, 0, sizeof(double) * std::max<long long>(1, A.creg_elems), st);
        cudaMemsetAsync(H->lev[l + 1].freg, 0, sizeof(double) * std::max<long long>(1, H->lev[l + 1].freg_elems), st);
    }
    if (fused_cfl(H, l)) {  // the estimate is the last substep's
        k_reset_cfl<<<1, 1, 0, st>>>(L->d_step);
        ++launches_counter;
    }
    for (int k = 0; k < R.nst && s == OCFD_OK; ++k) {
        double a[4];
        cf_coefs(R.order, k, theta, r, a);
        s = fill_level(H, l, L->buf[R.src[k]], a, R.tfrac[k], st);
        if (s == OCFD_OK) s = launch_stage(L, k, flags, st);
        launches_counter += stage_launches(L, flags);
    }
    if (s != OCFD_OK) return s;
    if (R.copy_out && cudaMemcpyAsync(L->buf[has_child ? 3 : 0], L->buf[1], sizeof(double) * L->elems,
                                      cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return check_launch("AMR stage output copy");
    if (has_child) {
        double a[4];
        cf_coefs(R.order, 3, theta, r, a);
        s = fill_level(H, l, L->buf[3], a, 1.0, st);
        for (int i = 1; i <= 2 && s == OCFD_OK; ++i) s = advance_level(H, l + 1, i, flags, st);
        if (s != OCFD_OK) return s;
        AmrLev& F = H->lev[l + 1];
        if (F.nrc > 0) {
            k_reflux<<<(F.nrc + 127) / 128, 128, 0, st>>>(F.d_rc, F.nrc, F.d_rf, A.creg, F.freg, L->buf[3],
                                                         1.0 / A.dx[0], 1.0 / A.dx[1], 1.0 / A.dx[2], L->ncomp);
            ++launches_counter;
        }
        s = launch_avg(H, l + 1, F.L->buf[0], L->buf[3], st);
        if (s != OCFD_OK) return s;
        if (cudaMemcpyAsync(L->buf[0], L->buf[3], sizeof(double) * L->elems, cudaMemcpyDeviceToDevice, st) !=
            cudaSuccess)
            return check_launch("AMR D -> A");
    }
    if (l > 0) {
        k_sub_end<<<1, 1, 0, st>>>(L->d_step);
        ++launches_counter;
    }
    return check_launch("AMR level advance");
}

// CFL estimates of every level from its state (all = false: the levels whose
// estimate the step's stages did not fuse)
static ocfd_status launch_estdt_all(ocfd_amr* H, cudaStream_t st, bool all = true) {
    for (int l = 0; l < H->nlev; ++l) {
        if (!all && fused_cfl(H, l)) continue;
        ocfd_level* L = H->lev[l].L;
        k_estdt_into<<<grid_for(L->ncells, 256, H->ctx->num_sms), 256, 0, st>>>(
            L->d_fabs, L->d_cell_start, (int)L->boxes.size(), L->ncells, L->buf[0], H->ctx->parm, L->desc.dx[0],
            L->desc.dx[1], L->desc.dx[2], &L->d_step->cfl_min);
        ++launches_counter;
    }
    return check_launch("AMR estdt");
}

static ocfd_status record_amr_step(ocfd_amr* H, unsigned flags, cudaStream_t st) {
    launches_counter = 0;
    k_amr_begin<<<1, 1, 0, st>>>(states(H));
    ocfd_status s = advance_level(H, 0, 1, flags, st);
    if (s == OCFD_OK && !H->react) s = launch_estdt_all(H, st, false);
    k_amr_end<<<1, 1, 0, st>>>(states(H));
    launches_counter += 2;
    H->launches = launches_counter;
    if (s != OCFD_OK) return s;
    return check_launch("AMR step");
}

// all levels' ghosts from their current state A, bottom-up
static ocfd_status fill_all_sync(ocfd_amr* H, cudaStream_t st) {
    const double a[4] = {1.0, 0.0, 0.0, 0.0};
    for (int l = 0; l < H->nlev; ++l) {
        ocfd_status s = fill_level(H, l, H->lev[l].L->buf[0], a, 0.0, st);
        if (s != OCFD_OK) return s;
    }
    return OCFD_OK;
}

// ---------------------------------------------------------------- regridding
struct BlockGrid {
    IBox dom;      // level domain (cells of the level)
    int bf[3];     // block size in cells of the level
    int nb[3];
    std::vector<unsigned char> v;
    size_t at(int i, int j, int k) const { return (size_t)i + (size_t)nb[0] * ((size_t)j + (size_t)nb[1] * k); }
};

static void block_geometry(const ocfd_amr* H, int f, BlockGrid& g) {
    g.dom = level_domain(H, f);
    for (int e = 0; e < 3; ++e) {
        const int ext = g.dom.hi[e] - g.dom.lo[e] + 1;
        g.bf[e] = std::min(H->desc.blocking_factor[e], ext);
        g.nb[e] = ext / g.bf[e];
    }
    g.v.assign((size_t)g.nb[0] * g.nb[1] * g.nb[2], 0);
}

static IBox block_box(const BlockGrid& g, int i, int j, int k) {
    const int b[3] = {i, j, k};
    IBox r;
    for (int e = 0; e < 3; ++e) {
        r.lo[e] = g.dom.lo[e] + b[e] * g.bf[e];
        r.hi[e] = r.lo[e] + g.bf[e] - 1;
    }
    return r;
}

// mark the blocks of g that meet region r (level cells; periodic images wrapped,
// non-periodic parts outside the domain dropped)
static void mark_region(const ocfd_amr* H, BlockGrid& g, const IBox& r) {
    std::vector<std::array<int, 3>> shifts;
    periodic_shifts(H, g.dom, shifts);
    for (const auto& sh : shifts) {
        IBox q;
        if (!ib_isect(ib_shift(r, sh.data()), g.dom, q)) continue;
        int lo[3], hi[3];
        for (int e = 0; e < 3; ++e) {
            lo[e] = (q.lo[e] - g.dom.lo[e]) / g.bf[e];
            hi[e] = (q.hi[e] - g.dom.lo[e]) / g.bf[e];
        }
        for (int k = lo[2]; k <= hi[2]; ++k)
            for (int j = lo[1]; j <= hi[1]; ++j)
                for (int i = lo[0]; i <= hi[0]; ++i) g.v[g.at(i, j, k)] = 1;
    }
}

// is region r (level cells) inside the boxes of `idx` wherever it is inside the domain?
static bool region_covered(const ocfd_amr* H, const BoxIndex& idx, const IBox& r) {
    std::vector<std::array<int, 3>> shifts;
    periodic_shifts(H, idx.dom, shifts);
    for (const auto& sh : shifts) {
        IBox q;
        if (!ib_isect(ib_shift(r, sh.data()), idx.dom, q)) continue;
        std::vector<IBox> rest{q};
        for (int b : idx.query(q)) {
            list_subtract(rest, idx.boxes[b]);
            if (rest.empty()) break;
        }
        if (!rest.empty()) return false;
    }
    return true;
}

static std::vector<IBox> cluster_blocks(const ocfd_amr* H, const BlockGrid& g) {
    std::vector<IBox> out;
    std::vector<unsigned char> used(g.v.size(), 0);
    int mg[3];
    for (int e = 0; e < 3; ++e) mg[e] = std::max(1, H->desc.max_grid_size[e] / g.bf[e]);
    auto ok = [&](int i, int j, int k) { return g.v[g.at(i, j, k)] && !used[g.at(i, j, k)]; };
    for (int k = 0; k < g.nb[2]; ++k)
        for (int j = 0; j < g.nb[1]; ++j)
            for (int i = 0; i < g.nb[0]; ++i) {
                if (!ok(i, j, k)) continue;
                int ex = 1, ey = 1, ez = 1;
                while (i + ex < g.nb[0] && ex < mg[0] && ok(i + ex, j, k)) ++ex;
                while (j + ey < g.nb[1] && ey < mg[1]) {
                    bool row = true;
                    for (int a = 0; a < ex && row; ++a) row = ok(i + a, j + ey, k);
                    if (!row) break;
                    ++ey;
                }
                while (k + ez < g.nb[2] && ez < mg[2]) {
                    bool pl = true;
                    for (int b = 0; b < ey && pl; ++b)
                        for (int a = 0; a < ex && pl; ++a) pl = ok(i + a, j + b, k + ez);
                    if (!pl) break;
                    ++ez;
                }
                for (int c = 0; c < ez; ++c)
                    for (int b = 0; b < ey; ++b)
                        for (int a = 0; a < ex; ++a) used[g.at(i + a, j + b, k + c)] = 1;
                IBox lo = block_box(g, i, j, k), hi = block_box(g, i + ex - 1, j + ey - 1, k + ez - 1);
                IBox r;
                for (int e = 0; e < 3; ++e) { r.lo[e] = lo.lo[e]; r.hi[e] = hi.hi[e]; }
                out.push_back(r);
            }
    return out;
}

static bool same_boxes(const std::vector<IBox>& a, const std::vector<IBox>& b) {
    if (a.size() != b.size()) return false;
    for (size_t i = 0; i < a.size(); ++i)
        if (!ib_same(a[i], b[i])) return false;
    return true;
}

static ocfd_status launch_copy(ocfd_amr* H, ocfd_level* dst, const std::vector<IBox>& dboxes, ocfd_level* src,
                               const std::vector<IBox>& sboxes, cudaStream_t st) {
    std::vector<CopyTag> tags;
    for (int d = 0; d < (int)dboxes.size(); ++d)
        for (int s = 0; s < (int)sboxes.size(); ++s) {
            IBox I;
            if (!ib_isect(dboxes[d], sboxes[s], I)) continue;
            CopyTag t{};
            t.dst = d;
            t.src = s;
            for (int e = 0; e < 3; ++e) { t.lo[e] = I.lo[e]; t.hi[e] = I.hi[e]; }
            tags.push_back(t);
        }
    if (tags.empty()) return OCFD_OK;
    DevTags<CopyTag> dt;
    ocfd_status s = dt.set(tags, &H->pool);
    if (s == OCFD_OK) {
        k_copy_tags<<<grid_for(dt.total, 256, H->ctx->num_sms), 256, 0, st>>>(
            dt.d, dt.start, dt.n, dt.total, dst->d_fabs, dst->buf[0], src->d_fabs, src->buf[0], dst->ncomp);
        ++launches_counter;
        s = check_launch("AMR regrid copy");
    }
    cudaStreamSynchronize(st);
    dt.release(&H->pool);
    return s;
}

// Install new grids for levels lbase+1 .. lbase+grids.size() (empty list ends the
// hierarchy); ghosts of levels <= lbase must hold the current state.
static ocfd_status apply_grids(ocfd_amr* H, int lbase, const std::vector<std::vector<IBox>>& grids, cudaStream_t st) {
    int newfinest = lbase;
    for (size_t q = 0; q < grids.size(); ++q) {
        if (grids[q].empty()) break;
        newfinest = lbase + 1 + (int)q;
    }
    if (newfinest >= OCFD_AMR_MAX_LEVELS || newfinest > H->desc.max_level)
        return fail(OCFD_BAD_ARG, "AMR: more levels than max_level");
    // unchanged hierarchy: tables and graph stay valid
    bool changed = newfinest != H->nlev - 1;
    for (int f = lbase + 1; f <= newfinest && !changed; ++f)
        changed = !(f < H->nlev && same_boxes(grids[f - lbase - 1], H->lev[f].boxes));
    if (!changed) return OCFD_OK;
    PhaseTimer pt;
    const double a[4] = {1.0, 0.0, 0.0, 0.0};
    for (int f = lbase + 1; f <= newfinest; ++f) {
        const std::vector<IBox>& nb = grids[f - lbase - 1];
        const bool exists = f < H->nlev;
        if (exists && same_boxes(nb, H->lev[f].boxes)) continue;
        ocfd_level* NL = nullptr;
        ocfd_status s = make_level(H, f, nb, f < newfinest ? 4 : 3, &NL);
        if (s != OCFD_OK) return s;
        pt.mark("  make level", st);
        AmrLev& A = H->lev[f];
        ocfd_level* old = exists ? A.L : nullptr;
        std::vector<IBox> oldboxes = exists ? A.boxes : std::vector<IBox>();
        A.release_tables(&H->pool);
        A.L = NL;
        A.boxes = nb;
        A.dom = level_domain(H, f);
        for (int e = 0; e < 3; ++e) A.dx[e] = H->desc.dx[e] / (double)(1 << f);
        if (H->nlev < f + 1) H->nlev = f + 1;
        // clock of level 0; the CFL estimate of the level it replaces (the step's dt
        // comes from the estimates made at the end of the previous step)
        k_copy_step<<<1, 1, 0, st>>>(NL->d_step, H->lev[0].L->d_step, old ? old->d_step : nullptr);
        ++launches_counter;
        // cells the old level did not cover from the level below, the rest copied
        {
            std::vector<std::vector<IBox>> regions(nb.size());
            for (size_t b = 0; b < nb.size(); ++b) {
                regions[b] = {nb[b]};
                for (const IBox& ob : oldboxes) {
                    IBox t;
                    if (ib_isect(nb[b], ob, t)) list_subtract(regions[b], ob);
                }
            }
            std::vector<CfTag> tags;
            s = build_cf_tags(H, f, regions, tags);
            if (s == OCFD_OK) s = A.cf.set(tags, &H->pool);
            if (s == OCFD_OK) s = launch_cf(H, f, NL->buf[0], a, st);
        }
        pt.mark("  interpolate new level", st);
        if (s == OCFD_OK && old) s = launch_copy(H, NL, nb, old, oldboxes, st);
        pt.mark("  copy old level", st);
        if (old) {
            cudaStreamSynchronize(st);
            ocfd_level_destroy(old);
        }
        if (s != OCFD_OK) return s;
        // ghosts of the new level (its finer neighbour interpolates from them)
        {
            std::vector<std::vector<IBox>> regions;
            ghost_regions(H, f, regions);
            std::vector<CfTag> tags;
            s = build_cf_tags(H, f, regions, tags);
            if (cudaStreamSynchronize(st) != cudaSuccess) return check_launch("AMR regrid");
            if (s == OCFD_OK) s = A.cf.set(tags, &H->pool);
            if (s == OCFD_OK) s = fill_level(H, f, NL->buf[0], a, 0.0, st);
            if (s != OCFD_OK) return s;
        }
        pt.mark("  destroy old + ghosts", st);
    }
    for (int f = newfinest + 1; f < H->nlev; ++f) {
        cudaStreamSynchronize(st);
        H->lev[f].release_tables(&H->pool);
        ocfd_level_destroy(H->lev[f].L);
        H->lev[f].L = nullptr;
        H->lev[f].boxes.clear();
    }
    H->nlev = newfinest + 1;
    // every level's clock follows level 0
    {
        AmrStates S = states(H);
        StepState h{};
        cudaStreamSynchronize(st);
        if (cudaMemcpy(&h, S.s[0], sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return check_launch("AMR time");
        for (int l = 1; l < H->nlev; ++l) {
            StepState q{};
            if (cudaMemcpy(&q, S.s[l], sizeof(q), cudaMemcpyDeviceToHost) != cudaSuccess) return check_launch("AMR time");
            const unsigned long long est = q.cfl_min;
            q = h;
            q.cfl_min = est;
            if (cudaMemcpy(S.s[l], &q, sizeof(q), cudaMemcpyHostToDevice) != cudaSuccess) return check_launch("AMR time");
        }
    }
    pt.mark("  clocks", st);
    ocfd_status r = rebuild_tables(H);
    pt.mark("  rebuild tables", st);
    return r;
}

static ocfd_status regrid_impl(ocfd_amr* H, int lbase, cudaStream_t st);

static ocfd_status regrid(ocfd_amr* H, int lbase, cudaStream_t st) {
    const int c0 = launches_counter;
    ocfd_status s = regrid_impl(H, lbase, st);
    H->kernel_total += launches_counter - c0;
    return s;
}

static ocfd_status regrid_impl(ocfd_amr* H, int lbase, cudaStream_t st) {
    if (lbase < 0 || lbase >= H->nlev) return fail(OCFD_BAD_ARG, "ocfd_amr_regrid: lbase");
    if (lbase >= H->desc.max_level) return OCFD_OK;
    PhaseTimer pt;
    ocfd_status s = fill_all_sync(H, st);
    if (s != OCFD_OK) return s;
    pt.mark("sync fill", st);
    const int top = std::min(H->nlev - 1, H->desc.max_level - 1);
    std::vector<BlockGrid> T(top + 2);
    for (int l = lbase; l <= top; ++l) {
        BlockGrid& g = T[l + 1];
        block_geometry(H, l + 1, g);
        AmrLev& A = H->lev[l];
        const long long nblk = (long long)g.v.size();
        if (A.nblk_cap < nblk) {
            cudaFree(A.d_blk);
            if (cudaMalloc(&A.d_blk, nblk) != cudaSuccess) {
                cudaGetLastError();
                return fail(OCFD_OUT_OF_MEMORY, "AMR tag blocks");
            }
            A.nblk_cap = nblk;
        }
        cudaMemsetAsync(A.d_blk, 0, nblk, st);
        TagGeom tg{};
        for (int e = 0; e < 3; ++e) {
            tg.dom_lo[e] = A.dom.lo[e];
            tg.dom_hi[e] = A.dom.hi[e];
            tg.bs[e] = g.bf[e] / 2;
            tg.nb[e] = g.nb[e];
        }
        tg.nbuf = H->desc.n_error_buf;
        tg.thr = H->desc.refine_dengrad;
        tg.zvirt = A.L->zvirt ? 1 : 0;
        ocfd_level* L = A.L;
        k_tag_dengrad<<<grid_for(L->ncells, 256, H->ctx->num_sms), 256, 0, st>>>(
            L->d_fabs, L->d_cell_start, (int)L->boxes.size(), L->ncells, L->buf[0], tg, A.d_blk);
        ++launches_counter;
        s = check_launch("AMR tagging");
        if (s != OCFD_OK) return s;
        if (cudaMemcpyAsync(g.v.data(), A.d_blk, nblk, cudaMemcpyDeviceToHost, st) != cudaSuccess)
            return check_launch("AMR tag download");
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) return check_launch("AMR tagging");
    pt.mark("tag + download", st);
    // top-down: a level also covers the neighbourhood of the new level above it
    for (int f = top + 1; f >= lbase + 2; --f) {
        BlockGrid& fine = T[f];
        BlockGrid& crse = T[f - 1];
        for (int k = 0; k < fine.nb[2]; ++k)
            for (int j = 0; j < fine.nb[1]; ++j)
                for (int i = 0; i < fine.nb[0]; ++i)
                    if (fine.v[fine.at(i, j, k)]) mark_region(H, crse, ib_grow(ib_coarsen(block_box(fine, i, j, k)), kNest));
    }
    // bottom-up: drop blocks not properly nested, cluster
    std::vector<std::vector<IBox>> grids;
    BoxIndex below;
    below.build(H->lev[lbase].boxes, H->lev[lbase].dom);
    for (int f = lbase + 1; f <= top + 1; ++f) {
        BlockGrid& g = T[f];
        for (int k = 0; k < g.nb[2]; ++k)
            for (int j = 0; j < g.nb[1]; ++j)
                for (int i = 0; i < g.nb[0]; ++i) {
                    unsigned char& v = g.v[g.at(i, j, k)];
                    if (v && !region_covered(H, below, ib_grow(ib_coarsen(block_box(g, i, j, k)), kNest))) v = 0;
                }
        std::vector<IBox> boxes = cluster_blocks(H, g);
        grids.push_back(boxes);
        if (boxes.empty()) break;
        below.build(boxes, g.dom);
    }
    pt.mark("cluster", st);
    s = apply_grids(H, lbase, grids, st);
    pt.mark("apply grids", st);
    return s;
}

static ocfd_status ensure_graph(ocfd_amr* H, unsigned flags) {
    if (H->graph_ok && H->graph && H->graph_flags == flags) return OCFD_OK;
    if (H->graph) {
        cudaGraphExecDestroy(H->graph);
        H->graph = nullptr;
    }
    PhaseTimer pt;
    cudaStream_t cap;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return check_launch("capture stream");
    cudaGraph_t g;
    if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaStreamDestroy(cap);
        return check_launch("begin capture");
    }
    ocfd_status s = record_amr_step(H, flags, cap);
    cudaError_t e = cudaStreamEndCapture(cap, &g);
    cudaStreamDestroy(cap);
    if (s != OCFD_OK) return s;
    if (e != cudaSuccess) return fail(OCFD_LAUNCH_FAIL, std::string("AMR end capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&H->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(OCFD_LAUNCH_FAIL, std::string("AMR graph instantiate: ") + cudaGetErrorString(e));
    H->graph_flags = flags;
    H->graph_ok = true;
    pt.mark("graph capture", 0);
    return OCFD_OK;
}

}  // namespace ocfd

using namespace ocfd;

extern "C" {

ocfd_status ocfd_amr_autotune(ocfd_amr* H, unsigned flags, int reps, void* stream) {
    if (!H || reps <= 0) return fail(OCFD_BAD_ARG, "ocfd_amr_autotune");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    for (int l = 0; l < H->nlev; ++l) {
        ocfd_status s = level_autotune(H->lev[l].L, flags & ~(unsigned)OCFD_PER_BOX, reps, st);
        if (s != OCFD_OK) return s;
        H->tuned_tile[l] = H->lev[l].L->tile;
        H->tuned_sched[l] = H->lev[l].L->sched;
    }
    H->graph_ok = false;
    return OCFD_OK;
}

int ocfd_amr_tuned(const ocfd_amr* H, int lev, int32_t* tile, int32_t* sched) {
    if (!H || lev < 0 || lev >= H->nlev) return -1;
    if (tile) *tile = H->lev[lev].L->tile;
    if (sched) *sched = H->lev[lev].L->sched;
    return 0;
}

ocfd_status ocfd_amr_set_time_integration(ocfd_amr* H, int32_t order) {
    if (!H || order < 1 || order > 3) return fail(OCFD_BAD_ARG, "ocfd_amr_set_time_integration: order is 1, 2 or 3");
    if (H->react && order == 3)
        return fail(OCFD_UNSUPPORTED, "ocfd_amr_set_time_integration: the reacting hierarchy steps with RK2 or Euler");
    if (order == H->rk_order) return OCFD_OK;
    if (cudaDeviceSynchronize() != cudaSuccess) return check_launch("ocfd_amr_set_time_integration");
    H->rk_order = order;
    for (int l = 0; l < H->nlev; ++l) H->lev[l].L->rk_order = order;
    return rebuild_tables(H);
}

ocfd_status ocfd_amr_set_eb(ocfd_amr* H, const ocfd_eb_desc* eb) {
    if (!H || !eb) return fail(OCFD_BAD_ARG, "ocfd_amr_set_eb: null argument");
    if (H->react && eb->kind != OCFD_EB_NONE)
        return fail(OCFD_UNSUPPORTED, "ocfd_amr_set_eb: the reacting hierarchy has no embedded body");
    if (cudaDeviceSynchronize() != cudaSuccess) return check_launch("ocfd_amr_set_eb");
    H->has_eb = eb->kind != OCFD_EB_NONE;
    H->eb = *eb;
    for (int l = 0; l < H->nlev; ++l) {
        ocfd_status s = eb_setup(H->lev[l].L, *eb);
        if (s == OCFD_OK) s = rebuild_fill_tags(H->lev[l].L);
        if (s != OCFD_OK) return s;
    }
    ocfd_status s = rebuild_tables(H);
    H->need_estdt = true;
    return s;
}

static ocfd_status amr_create(ocfd_context* ctx, const ocfd_amr_desc* desc, const ocfd_amr_react_desc* react,
                              ocfd_amr** out);

ocfd_status ocfd_amr_create(ocfd_context* ctx, const ocfd_amr_desc* desc, ocfd_amr** out) {
    return amr_create(ctx, desc, nullptr, out);
}

ocfd_status ocfd_amr_create_reacting(ocfd_context* ctx, const ocfd_amr_desc* desc, const ocfd_amr_react_desc* react,
                                     ocfd_amr** out) {
    if (!react) return fail(OCFD_BAD_ARG, "ocfd_amr_create_reacting: null react description");
    if (!(react->dt > 0) || react->chem_substeps < 0 || (react->flags & ~(unsigned)(OCFD_VISC | OCFD_FLUX_FP32)))
        return fail(OCFD_BAD_ARG, "ocfd_amr_create_reacting: dt > 0, chem_substeps >= 0, flags OCFD_VISC | OCFD_FLUX_FP32");
    return amr_create(ctx, desc, react, out);
}

static ocfd_status amr_create(ocfd_context* ctx, const ocfd_amr_desc* desc, const ocfd_amr_react_desc* react,
                              ocfd_amr** out) {
    if (!ctx || !desc || !out || desc->nbox0 <= 0 || !desc->boxes0) return fail(OCFD_BAD_ARG, "ocfd_amr_create: bad arguments");
    *out = nullptr;
    if (desc->max_level < 0 || desc->max_level >= OCFD_AMR_MAX_LEVELS)
        return fail(OCFD_BAD_ARG, "ocfd_amr_create: max_level out of range");
    for (int e = 0; e < 3; ++e) {
        const int ext = desc->domain.hi[e] - desc->domain.lo[e] + 1;
        if (ext <= 0 || desc->max_grid_size[e] <= 0 || desc->blocking_factor[e] <= 0)
            return fail(OCFD_BAD_ARG, "ocfd_amr_create: domain, blocking_factor and max_grid_size must be positive");
        for (int l = 1; l <= desc->max_level; ++l) {
            const int el = ext << l;
            const int bf = std::min(desc->blocking_factor[e], el);
            if (bf % 2 != 0 || el % bf != 0)
                return fail(OCFD_BAD_ARG, "ocfd_amr_create: blocking_factor must be even and divide every level's domain");
        }
    }
    if (desc->n_error_buf < 0) return fail(OCFD_BAD_ARG, "ocfd_amr_create: n_error_buf");
    ocfd_amr* H = new ocfd_amr();
    H->ctx = ctx;
    H->desc = *desc;
    if (react) {
        H->react = true;
        H->ncomp = 5 + NSP;
        H->rdesc = *react;
        H->rk_order = 2;  // the reference's multispecies flow step supports Euler and RK2 (FlowAdvance.cpp:49-88)
    }
    H->boxes0.assign(desc->boxes0, desc->boxes0 + desc->nbox0);
    H->desc.boxes0 = nullptr;
    for (int e = 0; e < 3; ++e) H->periodic[e] = desc->lo_bc[e] == OCFD_BC_INTERIOR;
    std::vector<IBox> b0;
    long long cells = 0;
    for (const ocfd_box& b : H->boxes0) {
        b0.push_back(ib_of(b));
        cells += ib_cells(ib_of(b));
    }
    if (cells != ib_cells(ib_of(desc->domain))) {
        delete H;
        return fail(OCFD_BAD_ARG, "ocfd_amr_create: level-0 boxes must cover the domain");
    }
    ocfd_level* L0 = nullptr;
    ocfd_status s = make_level(H, 0, b0, 3, &L0);
    if (s != OCFD_OK) {
        delete H;
        return s;
    }
    H->lev[0].L = L0;
    H->lev[0].boxes = b0;
    H->lev[0].dom = level_domain(H, 0);
    for (int e = 0; e < 3; ++e) H->lev[0].dx[e] = desc->dx[e];
    H->nlev = 1;
    s = rebuild_tables(H);
    if (s == OCFD_OK && cudaDeviceSynchronize() != cudaSuccess) s = check_launch("ocfd_amr_create");
    if (s != OCFD_OK) {
        ocfd_amr_destroy(H);
        return s;
    }
    *out = H;
    return OCFD_OK;
}

ocfd_status ocfd_amr_destroy(ocfd_amr* H) {
    if (!H) return OCFD_OK;
    cudaDeviceSynchronize();
    if (H->graph) cudaGraphExecDestroy(H->graph);
    for (int l = 0; l < OCFD_AMR_MAX_LEVELS; ++l) {
        H->lev[l].release_tables(&H->pool);
        cudaFree(H->lev[l].d_blk);
        if (H->lev[l].L) ocfd_level_destroy(H->lev[l].L);
    }
    delete H;
    return OCFD_OK;
}

int ocfd_amr_nlevels(const ocfd_amr* H) { return H ? H->nlev : 0; }

ocfd_level* ocfd_amr_level(ocfd_amr* H, int lev) {
    if (!H || lev < 0 || lev >= H->nlev) return nullptr;
    return H->lev[lev].L;
}

int ocfd_amr_get_grids(const ocfd_amr* H, int lev, ocfd_box* out, int cap) {
    if (!H || lev < 0 || lev >= H->nlev) return -1;
    const std::vector<IBox>& b = H->lev[lev].boxes;
    for (int i = 0; i < (int)b.size() && i < cap; ++i) out[i] = ob_of(b[i]);
    return (int)b.size();
}

ocfd_status ocfd_amr_regrid(ocfd_amr* H, int lbase, void* stream) {
    if (!H) return fail(OCFD_BAD_ARG, "ocfd_amr_regrid");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    ocfd_status s = regrid(H, lbase, st);
    if (s == OCFD_OK && cudaStreamSynchronize(st) != cudaSuccess) s = check_launch("ocfd_amr_regrid");
    return s;
}

ocfd_status ocfd_amr_set_grids(ocfd_amr* H, int nlev, const int32_t* nbox, const ocfd_box* boxes, void* stream) {
    if (!H || nlev < 1 || nlev - 1 > H->desc.max_level || (nlev > 1 && (!nbox || !boxes)))
        return fail(OCFD_BAD_ARG, "ocfd_amr_set_grids");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    std::vector<std::vector<IBox>> grids;
    long long q = 0;
    for (int l = 1; l < nlev; ++l) {
        if (nbox[l] <= 0) return fail(OCFD_BAD_ARG, "ocfd_amr_set_grids: empty level");
        std::vector<IBox> g;
        const IBox dom = level_domain(H, l);
        for (int i = 0; i < nbox[l]; ++i) {
            IBox b = ib_of(boxes[q++]), t;
            if (!ib_isect(b, dom, t) || !ib_same(b, t)) return fail(OCFD_BAD_ARG, "ocfd_amr_set_grids: box outside the domain");
            for (int e = 0; e < 3; ++e)
                if (b.lo[e] % 2 != 0 || (b.hi[e] + 1) % 2 != 0)
                    return fail(OCFD_BAD_ARG, "ocfd_amr_set_grids: fine boxes must coarsen by 2");
            g.push_back(b);
        }
        grids.push_back(g);
    }
    grids.push_back({});
    ocfd_status s = fill_all_sync(H, st);
    if (s == OCFD_OK) s = apply_grids(H, 0, grids, st);
    if (s == OCFD_OK && cudaStreamSynchronize(st) != cudaSuccess) s = check_launch("ocfd_amr_set_grids");
    return s;
}

ocfd_status ocfd_amr_average_down(ocfd_amr* H, void* stream) {
    if (!H) return fail(OCFD_BAD_ARG, "ocfd_amr_average_down");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    for (int f = H->nlev - 1; f >= 1; --f) {
        ocfd_status s = launch_avg(H, f, H->lev[f].L->buf[0], H->lev[f - 1].L->buf[0], st);
        if (s != OCFD_OK) return s;
    }
    H->need_estdt = true;
    return OCFD_OK;
}

ocfd_status ocfd_amr_fill_ghosts(ocfd_amr* H, void* stream) {
    if (!H) return fail(OCFD_BAD_ARG, "ocfd_amr_fill_ghosts");
    return fill_all_sync(H, static_cast<cudaStream_t>(stream));
}

ocfd_status ocfd_amr_advance(ocfd_amr* H, int nsteps, double cfl, unsigned flags, void* stream) {
    if (!H || nsteps < 0 || !(cfl > 0)) return fail(OCFD_BAD_ARG, "ocfd_amr_advance");
    if (flags & ~(unsigned)(OCFD_FLUX_FP32 | OCFD_PER_BOX | OCFD_GRAVITY))
        return fail(OCFD_BAD_ARG, "ocfd_amr_advance: flags (inviscid ideal gas only)");
    if (H->react && (flags & ~(unsigned)OCFD_FLUX_FP32))
        return fail(OCFD_BAD_ARG, "ocfd_amr_advance: a reacting hierarchy takes OCFD_FLUX_FP32 only");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    for (int i = 0; i < nsteps; ++i) {
        if (H->desc.regrid_int > 0 && H->steps > 0 && H->steps % H->desc.regrid_int == 0) {
            ocfd_status s = regrid(H, 0, st);
            if (s != OCFD_OK) return s;
        }
        if (cudaMemcpyAsync(&H->lev[0].L->d_step->cfl, &cfl, sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess)
            return check_launch("ocfd_amr_advance");
        if (H->need_estdt) {
            const int c0 = launches_counter;
            k_reset_cfl_all<<<1, 1, 0, st>>>(states(H));
            ++launches_counter;
            ocfd_status s = launch_estdt_all(H, st);
            if (s != OCFD_OK) return s;
            H->kernel_total += launches_counter - c0;
            H->need_estdt = false;
        }
        if (flags & OCFD_PER_BOX) {  // host-issued launches (the reference's execution model)
            const int graph_launches = H->launches;
            ocfd_status s = record_amr_step(H, flags, st);
            H->kernel_total += H->launches;
            H->launches = graph_launches;
            if (s != OCFD_OK) return s;
        } else {
            ocfd_status s = ensure_graph(H, flags);
            if (s != OCFD_OK) return s;
            if (cudaGraphLaunch(H->graph, st) != cudaSuccess) return check_launch("AMR graph launch");
            H->kernel_total += H->launches;
        }
        ++H->steps;
    }
    return OCFD_OK;
}

ocfd_status ocfd_amr_time(ocfd_amr* H, double* time, double* last_dt0, void* stream) {
    if (!H) return fail(OCFD_BAD_ARG, "ocfd_amr_time");
    return ocfd_level_time(H->lev[0].L, time, last_dt0, stream);
}

ocfd_status ocfd_amr_set_time(ocfd_amr* H, double time, void* stream) {
    if (!H) return fail(OCFD_BAD_ARG, "ocfd_amr_set_time");
    k_amr_sync<<<1, 1, 0, static_cast<cudaStream_t>(stream)>>>(states(H), time, 1);
    H->need_estdt = true;
    H->steps = 0;
    return check_launch("ocfd_amr_set_time");
}

ocfd_status ocfd_amr_set_stop_time(ocfd_amr* H, double stop_time, void* stream) {
    if (!H) return fail(OCFD_BAD_ARG, "ocfd_amr_set_stop_time");
    k_amr_stop<<<1, 1, 0, static_cast<cudaStream_t>(stream)>>>(states(H), stop_time);
    return check_launch("ocfd_amr_set_stop_time");
}

ocfd_status ocfd_amr_cell_steps(const ocfd_amr* H, int64_t* leaf, int64_t* all) {
    if (!H) return fail(OCFD_BAD_ARG, "ocfd_amr_cell_steps");
    int64_t a = 0, b = 0;
    for (int l = 0; l < H->nlev; ++l) {
        a += (int64_t)H->lev[l].leaf << l;
        b += (int64_t)H->lev[l].L->ncells << l;
    }
    if (leaf) *leaf = a;
    if (all) *all = b;
    return OCFD_OK;
}

int ocfd_amr_launches_per_step(const ocfd_amr* H) { return H ? H->launches : 0; }

ocfd_status ocfd_amr_write_plotfile(ocfd_amr* H, const char* dir, int32_t step, void* stream) {
    if (!H || !dir) return fail(OCFD_BAD_ARG, "ocfd_amr_write_plotfile");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaStreamSynchronize(st) != cudaSuccess) return check_launch("ocfd_amr_write_plotfile");
    StepState s0{};
    if (cudaMemcpy(&s0, H->lev[0].L->d_step, sizeof(s0), cudaMemcpyDeviceToHost) != cudaSuccess)
        return check_launch("ocfd_amr_write_plotfile");
    const double gm1 = H->ctx->host_parm.eos_gamma - 1.;
    const int ncomp = 9;
    static const char* names[ncomp] = {"rho", "xmom", "ymom", "zmom", "Eden", "ux", "uy", "uz", "pressure"};
    std::vector<std::vector<std::vector<double>>> data(H->nlev);
    std::vector<std::vector<const double*>> ptrs(H->nlev);
    std::vector<std::vector<ocfd_box>> boxes(H->nlev);
    std::vector<ocfd_plot_level> lv(H->nlev);
    for (int l = 0; l < H->nlev; ++l) {
        ocfd_level* L = H->lev[l].L;
        std::vector<double> host((size_t)L->elems);
        if (cudaMemcpy(host.data(), L->buf[0], sizeof(double) * L->elems, cudaMemcpyDeviceToHost) != cudaSuccess)
            return check_launch("ocfd_amr_write_plotfile");
        for (size_t b = 0; b < L->boxes.size(); ++b) {
            const FabGeom& f = L->fabs[b];
            const long long nc = (long long)(f.hi[0] - f.lo[0] + 1) * (f.hi[1] - f.lo[1] + 1) * (f.hi[2] - f.lo[2] + 1);
            std::vector<double> v((size_t)nc * ncomp);
            long long c = 0;
            for (int k = f.lo[2]; k <= f.hi[2]; ++k)
                for (int j = f.lo[1]; j <= f.hi[1]; ++j)
                    for (int i = f.lo[0]; i <= f.hi[0]; ++i, ++c) {
                        const long long q = fab_index_h(f, i, j, k);
                        double u[5];
                        for (int n = 0; n < 5; ++n) u[n] = host[q + n * f.ns];
                        for (int n = 0; n < 5; ++n) v[n * nc + c] = u[n];
                        v[5 * nc + c] = u[1] / u[0];
                        v[6 * nc + c] = u[2] / u[0];
                        v[7 * nc + c] = u[3] / u[0];
                        v[8 * nc + c] = gm1 * (u[4] - 0.5 / u[0] * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]));
                    }
            data[l].push_back(std::move(v));
            boxes[l].push_back(L->boxes[b]);
        }
        for (auto& v : data[l]) ptrs[l].push_back(v.data());
        lv[l].nbox = (int32_t)boxes[l].size();
        lv[l].boxes = boxes[l].data();
        lv[l].fabs = ptrs[l].data();
        for (int e = 0; e < 3; ++e) lv[l].dx[e] = H->lev[l].dx[e];
        lv[l].step = step << l;
    }
    double phi[3];
    for (int e = 0; e < 3; ++e)
        phi[e] = H->desc.prob_lo[e] + H->desc.dx[e] * (H->desc.domain.hi[e] - H->desc.domain.lo[e] + 1);
    return ocfd_plotfile_write(dir, H->nlev, lv.data(), ncomp, names, &H->desc.domain, H->desc.prob_lo, phi, 2,
                               s0.time);
}

size_t ocfd_amr_state_elems(const ocfd_amr* H, int lev) {
    if (!H || lev < 0 || lev >= H->nlev) return 0;
    return (size_t)H->lev[lev].L->elems;
}

ocfd_status ocfd_amr_copy_in(ocfd_amr* H, int lev, const double* buf, void* stream) {
    if (!H || lev < 0 || lev >= H->nlev || !buf) return fail(OCFD_BAD_ARG, "ocfd_amr_copy_in");
    ocfd_level* L = H->lev[lev].L;
    if (cudaMemcpyAsync(L->buf[0], buf, sizeof(double) * L->elems, cudaMemcpyDefault,
                        static_cast<cudaStream_t>(stream)) != cudaSuccess)
        return check_launch("ocfd_amr_copy_in");
    H->need_estdt = true;
    return OCFD_OK;
}

ocfd_status ocfd_amr_copy_out(ocfd_amr* H, int lev, double* buf, void* stream) {
    if (!H || lev < 0 || lev >= H->nlev || !buf) return fail(OCFD_BAD_ARG, "ocfd_amr_copy_out");
    ocfd_level* L = H->lev[lev].L;
    if (cudaMemcpyAsync(buf, L->buf[0], sizeof(double) * L->elems, cudaMemcpyDefault,
                        static_cast<cudaStream_t>(stream)) != cudaSuccess)
        return check_launch("ocfd_amr_copy_out");
    return OCFD_OK;
}

int64_t ocfd_amr_valid_elems(const ocfd_amr* H, int lev) {
    if (!H || lev < 0 || lev >= H->nlev) return 0;
    return (int64_t)H->lev[lev].L->ncells * H->lev[lev].L->ncomp;
}

ocfd_status ocfd_amr_copy_valid_in(ocfd_amr* H, int lev, const double* buf, void* stream) {
    if (!H || lev < 0 || lev >= H->nlev || !buf) return fail(OCFD_BAD_ARG, "ocfd_amr_copy_valid_in");
    ocfd_status s = level_copy_valid(H->lev[lev].L, const_cast<double*>(buf), true, static_cast<cudaStream_t>(stream));
    H->need_estdt = true;
    return s;
}

ocfd_status ocfd_amr_copy_valid_out(ocfd_amr* H, int lev, double* buf, void* stream) {
    if (!H || lev < 0 || lev >= H->nlev || !buf) return fail(OCFD_BAD_ARG, "ocfd_amr_copy_valid_out");
    return level_copy_valid(H->lev[lev].L, buf, false, static_cast<cudaStream_t>(stream));
}

int64_t ocfd_amr_kernels_launched(const ocfd_amr* H) { return H ? H->kernel_total : 0; }

}  // extern "C"
