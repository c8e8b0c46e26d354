// Fused right-hand side of a regular (uncut) box, ideal gas, FP64 form.
//
// Replaces the per-box kernel chain of EBR::compute_dSdt (Source/Advance.cpp:
// 231-329): c2prim over the grown box, then per direction flux_split (full
// grown box), reconstruction (WENO-Z, per face and component), compute_visc,
// and finally divop - fused into one launch (rhs_regular_kernel.cuh).
#include <cuda_runtime.h>

#include "rhs_regular_kernel.cuh"

namespace ocfd {

ocfd_status configure_rhs_regular() { return configure_all<double>(); }

bool regular_tile_fits(int tile, bool visc) { return tile_fits<double>(tile, visc); }

const TileShape kRegularTiles[] = {{8, 8, 8}, {8, 8, 4}, {16, 8, 4}, {16, 16, 2}, {32, 8, 2}, {16, 8, 2}};
const int kNumRegularTiles = sizeof(kRegularTiles) / sizeof(kRegularTiles[0]);

ocfd_status launch_rhs_regular(int tile, bool visc, const RegBoxArgs* d_boxes,
                               const int* d_tile_start, int nbox, const RegBoxArgs& single,
                               int ntiles, const DevParm& P, cudaStream_t st, int sched, unsigned* queue) {
    return launch_any<double>(tile, visc, d_boxes, d_tile_start, nbox, single, ntiles, P, st, sched, queue);
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
    a.has_flux = flux != nullptr ? FLUX_WRITE : 0;
    a.flux_w = 0.0;
    for (int d = 0; d < 3; ++d) {
        if (flux) a.flux[d] = view_of<double>(&flux[d]);
        a.lo[d] = bx.lo[d];
        a.hi[d] = bx.hi[d];
        a.dxinv[d] = dxinv[d];
        a.dxinv_f[d] = (float)dxinv[d];
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
    if (flags & ~(unsigned)(OCFD_VISC | OCFD_FLUX_FP32 | OCFD_GRAVITY))
        return fail(OCFD_BAD_ARG, "ocfd_rhs_regular_box_f64: unknown flags");
    if (flags & OCFD_FLUX_FP32) return rhs_regular_box_f32(ctx, S, dSdt, flux, bx, dxinv, flags, stream);
    DevParm P = ctx->parm;
    P.grav = (flags & OCFD_GRAVITY) ? kGravity : 0.0;
    const int n[3] = {bx.hi[0] - bx.lo[0] + 1, bx.hi[1] - bx.lo[1] + 1, bx.hi[2] - bx.lo[2] + 1};
    const int tile = pick_regular_tile(n, (flags & OCFD_VISC) != 0);
    RegBoxArgs a{};
    fill_regular_args(a, S, dSdt, flux, bx, dxinv, tile);
    const int ntiles = a.ntile[0] * a.ntile[1] * a.ntile[2];
    return launch_rhs_regular(tile, (flags & OCFD_VISC) != 0, nullptr, nullptr, 1, a, ntiles,
                              P, static_cast<cudaStream_t>(stream));
}
