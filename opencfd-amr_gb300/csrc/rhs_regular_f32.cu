// Mixed-precision regular-box right-hand side (OCFD_FLUX_FP32): the kernel of
// rhs_regular_kernel.cuh instantiated with FP32 primitives, split, WENO-Z,
// viscous flux and divergence; FP64 state and RK accumulation.
#include <cuda_runtime.h>

#include "rhs_regular_kernel.cuh"

namespace ocfd {

ocfd_status configure_rhs_regular_f32() { return configure_all<float>(); }

ocfd_status launch_rhs_regular_f32(int tile, bool visc, const RegBoxArgs* d_boxes,
                               const int* d_tile_start, int nbox, const RegBoxArgs& single,
                               int ntiles, const DevParm& P, cudaStream_t st, int sched, unsigned* queue) {
    return launch_any<float>(tile, visc, d_boxes, d_tile_start, nbox, single, ntiles, P, st, sched, queue);
}

ocfd_status rhs_regular_box_f32(ocfd_context* ctx, const ocfd_array4* S, const ocfd_array4* dSdt,
                                const ocfd_array4* flux, const ocfd_box& bx,
                                const double dxinv[3], unsigned flags, void* stream) {
    const int n[3] = {bx.hi[0] - bx.lo[0] + 1, bx.hi[1] - bx.lo[1] + 1, bx.hi[2] - bx.lo[2] + 1};
    const bool visc = (flags & OCFD_VISC) != 0;
    int tile = pick_regular_tile(n, visc);
    if (!tile_fits<float>(tile, visc)) tile = 1;
    if (!visc) tile = staged_regular_tile(tile);  // TMA staging where the shape has it
    RegBoxArgs a{};
    fill_regular_args(a, S, dSdt, flux, bx, dxinv, tile);
    const int ntiles = a.ntile[0] * a.ntile[1] * a.ntile[2];
    DevParm P = ctx->parm;
    P.grav = (flags & OCFD_GRAVITY) ? kGravity : 0.0;
    return launch_any<float>(tile, visc, nullptr, nullptr, 1, a, ntiles, P, static_cast<cudaStream_t>(stream));
}

}  // namespace ocfd
