// Regular-box right-hand side: launch interface shared by the per-box C ABI
// entry point, the level driver and the batched (box-list) form.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "ocfd_internal.h"

namespace ocfd {

enum RhsMode { RHS_WRITE_DSDT = 0, RHS_FUSED_STAGE = 1 };
// tile schedules of the batched launch (k_rhs_regular)
enum TileSched { SCHED_GRID = 0, SCHED_STRIDE = 1, SCHED_QUEUE = 2, NUM_SCHED = 3 };
enum FluxBits { FLUX_WRITE = 1, FLUX_ACC_ALL = 2, FLUX_ACC_PLANES = 4 };

struct TileShape {
    int x, y, z;
    int staged;  // the TMA-staged variant of the shape (FP32-flux form, inviscid)
};
extern const TileShape kRegularTiles[];
extern const int kNumRegularTiles;

// Everything one box needs; a device array of these drives the batched form.
struct RegBoxArgs {
    View<const double> S;      // state with ghosts (stage input U_s)
    View<double> dsdt;         // RHS_WRITE_DSDT: output over the box
    View<double> flux[3];      // optional face-flux output
    // face-flux output, bit flags:
    //   FLUX_WRITE       flux[d] = F on every face of the box (per-box entry points)
    //   FLUX_ACC_ALL     flux[d] += flux_w * dt * F on every face (coarse side of a
    //                    flux register: time-weighted stage fluxes summed over RK3)
    //   FLUX_ACC_PLANES  fplane[d][side] += flux_w * dt * F on the box's own lo / hi
    //                    faces in d (fine side of a flux register)
    int has_flux;
    double flux_w;
    View<double> fplane[3][2];
    int lo[3], hi[3];
    double dxinv[3];
    float dxinv_f[3], dx_f[3];  // FP32 copies for the mixed form
    int ntile[3];
    int mode;
    // RHS_FUSED_STAGE: Uout = rk_a * U0 + rk_b * (S + dt * L(S)) over the box,
    // dt read from *dt_ptr when set (device-resident step size)
    View<const double> U0;
    View<double> Uout;
    double rk_a, rk_b, dt;
    const double* dt_ptr;
    // optional CFL reduction over the new state (Source/Advance.cpp:10-59):
    // atomicMin of min(dx_d / (|u_d| + c)) as ordered double bits
    unsigned long long* cfl_min;
    double dx[3];
    // z faces whose outside ghost cells are not filled (their BC takes values from
    // inside the domain): stencil loads read the source cell instead - the
    // boundary cell (foextrap) or the mirror cell (reflect) with the velocity
    // components of zsign (bit 0/1/2 = u/v/w) negated
    int zvirt;
    int zdom[2];
    int zmirror[2];
    int zsign[2];
    // TMA staging of a tile's cross (the FP32-flux form on tiles of depth >= 4):
    // tiled tensor maps of S as a 4-D tensor (x, y, z, component) whose boxes are
    // the tile's centre (TX x TY x TZ), x halo (4 x TY x TZ: the low one starts 4
    // cells before the tile, keeping every x offset even), y halo (TX x 3 x TZ)
    // and z halo (TX x TY x 3), 5 components each.  use_tma = 0 when S does not
    // meet TMA's rules (16-byte base and strides, even x offset of the box) or
    // the tile is not staged this way: the kernel then loads the cross with
    // plain loads, to the same values.
    CUtensorMap tmap[4];
    int use_tma;
};

// the cell a load at z index gk reads, and the velocity signs to flip
__host__ __device__ __forceinline__ int zmap(const RegBoxArgs& B, int gk, int& sign) {
    sign = 0;
    if (!B.zvirt) return gk;
    if (gk < B.zdom[0]) {
        sign = B.zsign[0];
        return B.zmirror[0] ? 2 * B.zdom[0] - 1 - gk : B.zdom[0];
    }
    if (gk > B.zdom[1]) {
        sign = B.zsign[1];
        return B.zmirror[1] ? 2 * B.zdom[1] + 1 - gk : B.zdom[1];
    }
    return gk;
}

// CFL bound dx/(|u|+c) of one conserved state, Source/Advance.cpp:26-49
__device__ __forceinline__ double cfl_bound(const DevParm& P, const double* u, const double* dx) {
    double rho = u[0];
    double rhoinv = 1.0 / (rho > P.smallr ? rho : P.smallr);
    double vx = u[1] * rhoinv, vy = u[2] * rhoinv, vz = u[3] * rhoinv;
    double pe = (P.gamma - 1.0) * (u[4] - 0.5 * rho * (vx * vx + vy * vy + vz * vz));
    double p = pe > P.smallp ? pe : P.smallp;
    double cs = sqrt(P.gamma * p * rhoinv);
    double dtx = dx[0] / (fabs(vx) + cs);
    double dty = dx[1] / (fabs(vy) + cs);
    double dtz = dx[2] / (fabs(vz) + cs);
    double m = dty < dtz ? dty : dtz;
    return dtx < m ? dtx : m;
}

// block-wide min of v (all threads participate; the block is whole warps, at
// most 1024 threads), one atomicMin per block
__device__ __forceinline__ void block_min_atomic(double v, unsigned long long* target) {
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) {
        double w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w < v ? w : v;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        v = lane < nw ? red[lane] : __longlong_as_double(0x7FF0000000000000LL);
        for (int o = 16; o > 0; o >>= 1) {
            double w = __shfl_xor_sync(0xffffffffu, v, o);
            v = w < v ? w : v;
        }
        if (lane == 0 && v >= 0.0) atomicMin(target, (unsigned long long)__double_as_longlong(v));
    }
}

// The CFL bound over many cells, min over cells of min_d dx_d / (|v_d| + c)
// (Source/Advance.cpp:26-49), kept as the three largest signal speeds
// s_d = |v_d| + c: correctly rounded division is monotone in the divisor, so the
// minimum over cells of dx_d / s_d is exactly dx_d / max s_d, and a block divides
// three times instead of three times per cell (GB300's FP64 pipe executes the
// divisions).  The speeds follow the reference's expression with every rounding
// written out (no contraction), so the bound is the correctly rounded value of
// that expression on any host or device.
struct CflSpeeds {
    double s[3] = {0.0, 0.0, 0.0};
    __device__ __forceinline__ void add(const DevParm& P, const double* u) {
        const double rho = u[0];
        const double rhoinv = __ddiv_rn(1.0, rho > P.smallr ? rho : P.smallr);
        const double vx = __dmul_rn(u[1], rhoinv), vy = __dmul_rn(u[2], rhoinv), vz = __dmul_rn(u[3], rhoinv);
        const double ke = __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz));
        const double pe = __dmul_rn(__dsub_rn(P.gamma, 1.0), __dsub_rn(u[4], __dmul_rn(__dmul_rn(0.5, rho), ke)));
        const double p = pe > P.smallp ? pe : P.smallp;
        const double cs = __dsqrt_rn(__dmul_rn(__dmul_rn(P.gamma, p), rhoinv));
        s[0] = fmax(s[0], __dadd_rn(fabs(vx), cs));
        s[1] = fmax(s[1], __dadd_rn(fabs(vy), cs));
        s[2] = fmax(s[2], __dadd_rn(fabs(vz), cs));
    }
};

// block-wide CFL bound from the threads' largest speeds (all threads
// participate; the block is whole warps, at most 1024 threads), one atomicMin
// per block; a block without cells adds +inf
__device__ __forceinline__ void block_cfl_atomic(const CflSpeeds& c, const double* dx, unsigned long long* target) {
    __shared__ double red[3][32];
    double s0 = c.s[0], s1 = c.s[1], s2 = c.s[2];
    for (int o = 16; o > 0; o >>= 1) {
        s0 = fmax(s0, __shfl_xor_sync(0xffffffffu, s0, o));
        s1 = fmax(s1, __shfl_xor_sync(0xffffffffu, s1, o));
        s2 = fmax(s2, __shfl_xor_sync(0xffffffffu, s2, o));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        red[0][warp] = s0;
        red[1][warp] = s1;
        red[2][warp] = s2;
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        s0 = lane < nw ? red[0][lane] : 0.0;
        s1 = lane < nw ? red[1][lane] : 0.0;
        s2 = lane < nw ? red[2][lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            s0 = fmax(s0, __shfl_xor_sync(0xffffffffu, s0, o));
            s1 = fmax(s1, __shfl_xor_sync(0xffffffffu, s1, o));
            s2 = fmax(s2, __shfl_xor_sync(0xffffffffu, s2, o));
        }
        if (lane == 0) {
            const double tx = dx[0] / s0, ty = dx[1] / s1, tz = dx[2] / s2;
            const double m = ty < tz ? ty : tz;
            const double v = tx < m ? tx : m;
            if (v >= 0.0) atomicMin(target, (unsigned long long)__double_as_longlong(v));
        }
    }
}

// g of the gravity source, Source/Advance.cpp:332
constexpr double kGravity = -9.8;

int pick_regular_tile(const int n[3], bool visc);
// the TMA-staged variant of tile's shape, or tile itself when it has none
int staged_regular_tile(int tile);
bool regular_tile_fits(int tile, bool visc);
ocfd_status configure_rhs_regular();
ocfd_status configure_rhs_regular_f32();
void fill_regular_args(RegBoxArgs& a, const ocfd_array4* S, const ocfd_array4* dSdt,
                       const ocfd_array4* flux, const ocfd_box& bx, const double dxinv[3],
                       int tile);
// tensor maps of a.tmap for S and `tile` (sets a.use_tma); false when S does not
// meet TMA's alignment rules or the driver entry point is missing
bool encode_regular_tmaps(RegBoxArgs& a, const ocfd_array4* S, int tile);
// process-wide switch of the TMA staging (tables built while it is off use
// plain loads); a test hook: both ways give the same results
void set_regular_tma(bool on);

// d_boxes == nullptr: one box given by `single`, ntiles CTAs.
// otherwise: nbox boxes, d_tile_start[b] = first CTA of box b, ntiles in total.
// sched / queue: TileSched and, for SCHED_QUEUE, two zeroed device words
ocfd_status launch_rhs_regular(int tile, bool visc, const RegBoxArgs* d_boxes,
                               const int* d_tile_start, int nbox, const RegBoxArgs& single,
                               int ntiles, const DevParm& P, cudaStream_t st, int sched = SCHED_GRID,
                               unsigned* queue = nullptr);
ocfd_status launch_rhs_regular_f32(int tile, bool visc, const RegBoxArgs* d_boxes,
                                   const int* d_tile_start, int nbox, const RegBoxArgs& single,
                                   int ntiles, const DevParm& P, cudaStream_t st, int sched = SCHED_GRID,
                                   unsigned* queue = nullptr);

ocfd_status rhs_regular_box_f32(ocfd_context* ctx, const ocfd_array4* S, const ocfd_array4* dSdt,
                                const ocfd_array4* flux, const ocfd_box& bx,
                                const double dxinv[3], unsigned flags, void* stream);

}  // namespace ocfd
