// Regular-box right-hand side: launch interface shared by the per-box C ABI
// entry point, the level driver and the batched (box-list) form.
#pragma once

#include <cuda_runtime.h>

#include "ocfd_internal.h"

namespace ocfd {

enum RhsMode { RHS_WRITE_DSDT = 0, RHS_FUSED_STAGE = 1 };

struct TileShape {
    int x, y, z;
};
extern const TileShape kRegularTiles[];
extern const int kNumRegularTiles;

// Everything one box needs; a device array of these drives the batched form.
struct RegBoxArgs {
    View<const double> S;      // state with ghosts (stage input U_s)
    View<double> dsdt;         // RHS_WRITE_DSDT: output over the box
    View<double> flux[3];      // optional face-flux output
    int has_flux;
    int lo[3], hi[3];
    double dxinv[3];
    int ntile[3];
    int mode;
    // RHS_FUSED_STAGE: Uout = rk_a * U0 + rk_b * (S + dt * L(S)) over the box
    View<const double> U0;
    View<double> Uout;
    double rk_a, rk_b, dt;
};

int pick_regular_tile(const int n[3]);
void fill_regular_args(RegBoxArgs& a, const ocfd_array4* S, const ocfd_array4* dSdt,
                       const ocfd_array4* flux, const ocfd_box& bx, const double dxinv[3],
                       int tile);

// d_boxes == nullptr: one box given by `single`, ntiles CTAs.
// otherwise: nbox boxes, d_tile_start[b] = first CTA of box b, ntiles in total.
ocfd_status launch_rhs_regular(int tile, bool visc, const RegBoxArgs* d_boxes,
                               const int* d_tile_start, int nbox, const RegBoxArgs& single,
                               int ntiles, const DevParm& P, cudaStream_t st);
ocfd_status launch_rhs_regular_f32(int tile, bool visc, const RegBoxArgs* d_boxes,
                                   const int* d_tile_start, int nbox, const RegBoxArgs& single,
                                   int ntiles, const DevParm& P, cudaStream_t st);

ocfd_status rhs_regular_box_f32(ocfd_context* ctx, const ocfd_array4* S, const ocfd_array4* dSdt,
                                const ocfd_array4* flux, const ocfd_box& bx,
                                const double dxinv[3], unsigned flags, void* stream);

}  // namespace ocfd
