// Fused right-hand side of a regular (uncut) box, ideal gas, FP64 form.
//
// Replaces the per-box kernel chain of EBR::compute_dSdt (Source/Advance.cpp:
// 231-329): c2prim over the grown box, then per direction flux_split (full
// grown box), reconstruction (WENO-Z, per face and component), compute_visc,
// and finally divop - fused into one launch (rhs_regular_kernel.cuh).
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include "rhs_regular_kernel.cuh"

namespace ocfd {

ocfd_status configure_rhs_regular() { return configure_all<double>(); }

bool regular_tile_fits(int tile, bool visc) { return tile_fits<double>(tile, visc); }

const TileShape kRegularTiles[] = {{8, 8, 8, 0},  {8, 8, 4, 0}, {16, 8, 4, 0}, {16, 16, 2, 0}, {32, 8, 2, 0},
                                   {16, 8, 2, 0}, {8, 8, 8, 1}, {8, 8, 4, 1}, {16, 8, 4, 1}};
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
        if (!regular_tile_fits(t, visc) || kRegularTiles[t].staged) continue;
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
    encode_regular_tmaps(a, S, tile);
}

int staged_regular_tile(int tile) {
    const TileShape& s = kRegularTiles[tile];
    for (int t = 0; t < kNumRegularTiles; ++t)
        if (kRegularTiles[t].staged && kRegularTiles[t].x == s.x && kRegularTiles[t].y == s.y &&
            kRegularTiles[t].z == s.z)
            return t;
    return tile;
}

static bool g_regular_tma = true;

void set_regular_tma(bool on) { g_regular_tma = on; }

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library); null when the driver does not offer it
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// The four box shapes of a tile's cross (centre, x halo 4 wide, y halo 3 deep,
// z halo 3 deep) over S as a (x, y, z, component) tensor of doubles.  TMA wants
// a 16-byte aligned base, strides that are multiples of 16 bytes and an x
// offset times 8 bytes that is a multiple of 16 for every box: the tiles start
// at lo + t TX with TX even and the x halo box at 4 cells before a tile, so
// (lo - begin) must be even.  Only tiles of depth >= 4 are staged this way.
bool encode_regular_tmaps(RegBoxArgs& a, const ocfd_array4* S, int tile) {
    a.use_tma = 0;
    if (!g_regular_tma || !S || tile < 0 || tile >= kNumRegularTiles) return false;
    const TileShape& t = kRegularTiles[tile];
    if (!t.staged || t.z < 4 || t.x % 2 != 0 || S->ncomp < 5) return false;
    const uintptr_t base = reinterpret_cast<uintptr_t>(S->p);
    if (base % 16 != 0 || S->jstride % 2 != 0 || S->kstride % 2 != 0 || S->nstride % 2 != 0) return false;
    if (((a.lo[0] - S->begin[0]) & 1) != 0) return false;
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dim[4] = {(cuuint64_t)(S->end[0] - S->begin[0]), (cuuint64_t)(S->end[1] - S->begin[1]),
                               (cuuint64_t)(S->end[2] - S->begin[2]), 5};
    const cuuint64_t stride[3] = {(cuuint64_t)S->jstride * 8, (cuuint64_t)S->kstride * 8,
                                  (cuuint64_t)S->nstride * 8};
    const cuuint32_t box[4][4] = {{(cuuint32_t)t.x, (cuuint32_t)t.y, (cuuint32_t)t.z, 5},
                                  {4, (cuuint32_t)t.y, (cuuint32_t)t.z, 5},
                                  {(cuuint32_t)t.x, 3, (cuuint32_t)t.z, 5},
                                  {(cuuint32_t)t.x, (cuuint32_t)t.y, 3, 5}};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    for (int m = 0; m < 4; ++m) {
        if (enc(&a.tmap[m], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, S->p, dim, stride, box[m], estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return false;
    }
    a.use_tma = 1;
    return true;
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

extern "C" void ocfd_set_tma_staging(int32_t on) { ocfd::set_regular_tma(on != 0); }
