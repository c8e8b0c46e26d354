// Level driver: box table, device ghost fill, fused RK steps in a CUDA graph.
//
// Storage: three state buffers A, B, C holding every box's FAB (box grown by
// NUM_GROW, components slowest, i fastest), boxes back to back.  An SSP-RK3
// step (the default) is
//   k_step_begin          dt = min(cfl * CFLmin, 1.1 dt_prev)  (device)
//   fill(A, t)      stage 1: B = A + dt L(A)
//   fill(B, t+dt)   stage 2: C = 3/4 A + 1/4 (B + dt L(B))
//   fill(C, t+dt/2) stage 3: A = 1/3 A + 2/3 (C + dt L(C))   + CFLmin of the new A
//   k_step_end            t += dt
// which is the Shu-Osher form of the SSP-RK3 that AmrLevel::RK(3, ...) runs
// (Source/Advance.cpp:141-148), with the stage times AMReX's RK3 fills ghosts
// at (t, t+dt, t+dt/2).  RK2 (Heun) and Euler, the other ebr.time_integration
// schemes (Source/Advance.cpp:115-138), are the two- and one-stage rows of the
// same table (rk_scheme).
//
// Ghost fill = same-level exchange (incl. periodic images; AMReX FillBoundary)
// followed by one pass per direction over the ghost cells outside the domain,
// x then y then z, applying the BC types of Source/Setup.cpp:17-92 per
// component and then the case functor (e.g. Exec/1_DMR/prob_bcfill.cpp).
// Pass d covers cells outside the domain in d, the grown range in directions
// before d and the in-domain range in directions after d, so edges and corners
// are filled from values set by earlier passes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "level.h"
#include "eb_level.h"

namespace ocfd {

__global__ void k_exchange(const ExTag* __restrict__ tags, const long long* __restrict__ start,
                           const int* __restrict__ chunk, int ntag, long long total,
                           const FabGeom* __restrict__ fabs, double* U, int ncomp) {
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int t = find_tag_chunked(start, chunk, ntag, idx);
        const ExTag& T = tags[t];
        int i, j, k;
        region_cell(T.lo, T.hi, idx - start[t], i, j, k);
        const FabGeom& fd = fabs[T.dst];
        const FabGeom& fs = fabs[T.src];
        const long long d = fab_index(fd, i, j, k);
        const long long s = fab_index(fs, i + T.shift[0], j + T.shift[1], k + T.shift[2]);
        for (int n = 0; n < ncomp; ++n) U[d + n * fd.ns] = U[s + n * fs.ns];
    }
}

// BC type codes (AMReX BCType): int_dir 0, ext_dir 1, foextrap 2, reflect_even 3, reflect_odd 4
__device__ __forceinline__ int bc_type(int phys, int comp, int d) {
    // Source/Setup.cpp:22-35 tables, rows Interior..NoSlipWall
    const int scalar[6] = {0, 1, 2, 3, 3, 3};
    const int normal[6] = {0, 1, 2, 4, 4, 4};
    const int tang[6] = {0, 1, 2, 3, 3, 4};
    if (comp >= 1 && comp <= 3) return (comp - 1 == d) ? normal[phys] : tang[phys];
    return scalar[phys];
}

// Exec/1_DMR/prob_bcfill.cpp:14-58 (x0 uses sin(pi/3) for amrex::Math::sinpi(1/3))
__device__ void dmr_functor(const BcInfo& bc, double* U, const FabGeom& f, long long c, int i,
                            int j, int k, int ncomp, double time) {
    const double x = bc.prob_lo[0] + (i + 0.5) * bc.dx[0];
    const double x0 = 1.0 / 6.0 + sqrt(1 / 3.0) + time * 10.0 / sin(3.14159265358979323846 * (1.0 / 3.0));
    const double* left = bc.params;
    const double* right = bc.params + 5;
    if (bc.hi_bc[1] == OCFD_BC_INFLOW && j > bc.dom_hi[1]) {
        const double* st = x < x0 ? left : right;
        for (int n = 0; n < ncomp && n < 5; ++n) U[c + n * f.ns] = st[n];
    }
    if ((bc.lo_bc[1] == 3 || bc.lo_bc[1] == 4 || bc.lo_bc[1] == 5) && j < bc.dom_lo[1]) {
        if (x < 1.0 / 6.0)
            for (int n = 0; n < ncomp && n < 5; ++n) U[c + n * f.ns] = left[n];
    }
    if (bc.lo_bc[0] == OCFD_BC_INFLOW && i < bc.dom_lo[0])
        for (int n = 0; n < ncomp && n < 5; ++n) U[c + n * f.ns] = left[n];
}

// Planar jet inflow on the x-lo face: with s(y) = (1 + tanh((w - |y - yc|) /
// delta)) / 2, u = u_co + (u_jet - u_co) s and rho = rho_co + (rho_jet - rho_co) s
// at uniform pressure (internal energy rho e); params = rho_jet, u_jet, u_co, yc,
// w, delta, rho e, rho_co
__device__ void jet_inflow(const BcInfo& bc, double* U, const FabGeom& f, long long c, int j, int ncomp) {
    const double* pr = bc.params;
    const double y = bc.prob_lo[1] + (j + 0.5) * bc.dx[1];
    const double s = 0.5 * (1.0 + tanh((pr[4] - fabs(y - pr[3])) / pr[5]));
    const double u = pr[2] + (pr[1] - pr[2]) * s;
    const double r = pr[7] + (pr[0] - pr[7]) * s;
    const double st[5] = {r, r * u, 0.0, 0.0, pr[6] + 0.5 * r * u * u};
    for (int n = 0; n < ncomp && n < 5; ++n) U[c + n * f.ns] = st[n];
}

template <int D>
__global__ void k_physbc(const BcTag* __restrict__ tags, const long long* __restrict__ start,
                         const int* __restrict__ chunk, int ntag, long long total,
                         const FabGeom* __restrict__ fabs, double* U, int ncomp, BcInfo bc,
                         const StepState* st, double tfrac) {
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int t = find_tag_chunked(start, chunk, ntag, idx);
        const BcTag& T = tags[t];
        int c3[3];
        region_cell(T.lo, T.hi, idx - start[t], c3[0], c3[1], c3[2]);
        const FabGeom& f = fabs[T.box];
        const long long c = fab_index(f, c3[0], c3[1], c3[2]);
        const int phys = T.side == 0 ? bc.lo_bc[D] : bc.hi_bc[D];
        for (int n = 0; n < ncomp; ++n) {
            const int ty = bc_type(phys, n, D);
            int s3[3] = {c3[0], c3[1], c3[2]};
            double sign = 1.0;
            if (ty == 2) {
                s3[D] = T.side == 0 ? bc.dom_lo[D] : bc.dom_hi[D];
            } else if (ty == 3 || ty == 4) {
                s3[D] = T.side == 0 ? 2 * bc.dom_lo[D] - 1 - c3[D] : 2 * bc.dom_hi[D] + 1 - c3[D];
                if (ty == 4) sign = -1.0;
            } else {
                continue;  // ext_dir: the case functor sets it; int_dir: exchange did
            }
            U[c + n * f.ns] = sign * U[fab_index(f, s3[0], s3[1], s3[2]) + n * f.ns];
        }
        if (bc.bc_case == OCFD_CASE_DMR) {
            const double time = st->time + tfrac * st->dt;
            dmr_functor(bc, U, f, c, c3[0], c3[1], c3[2], ncomp, time);
        } else if (bc.bc_case == OCFD_CASE_INFLOW) {
            if ((T.side == 0 ? bc.lo_bc[D] : bc.hi_bc[D]) == OCFD_BC_INFLOW)
                for (int n = 0; n < ncomp && n < 5; ++n) U[c + n * f.ns] = bc.params[n];
        } else if (bc.bc_case == OCFD_CASE_JET) {
            if (D == 0 && T.side == 0 && bc.lo_bc[0] == OCFD_BC_INFLOW) jet_inflow(bc, U, f, c, c3[1], ncomp);
        }
    }
}

__global__ void k_estdt(const FabGeom* __restrict__ fabs, const long long* __restrict__ start,
                        int nbox, long long total, const double* __restrict__ U, DevParm P,
                        double dx0, double dx1, double dx2, unsigned long long* out) {
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

__global__ void k_step_begin(StepState* st) {
    const double est = __longlong_as_double((long long)st->cfl_min);
    double dt = st->cfl * est;
    if (st->dt_prev > 0 && dt > 1.1 * st->dt_prev) dt = 1.1 * st->dt_prev;
    // stop-time limit of EBR::computeNewDt (Source/EBR.cpp:277-286): eps = 0.001 dt
    if (st->time + dt > st->stop_time - 0.001 * dt) dt = st->stop_time - st->time;
    if (dt < 0) dt = 0;
    st->dt = dt;
    st->cfl_min = 0x7FF0000000000000ULL;
}

__global__ void k_step_end(StepState* st) {
    st->time += st->dt;
    st->dt_prev = st->dt;
}

__global__ void k_reset_cfl(StepState* st) { st->cfl_min = 0x7FF0000000000000ULL; }

__global__ void k_set_stop(StepState* st, double t) { st->stop_time = t; }

__global__ void k_set_time(StepState* st, double t) {
    st->time = t;
    st->dt = 0;
    st->dt_prev = -1.0;
    st->cfl_min = 0x7FF0000000000000ULL;
}

int grid_for(long long total, int threads, int sms) {
    long long b = (total + threads - 1) / threads;
    long long cap = (long long)sms * 16;
    return (int)std::max<long long>(1, std::min(b, cap));
}

}  // namespace ocfd

using namespace ocfd;

namespace ocfd {

bool intersect(const int* alo, const int* ahi, const int* blo, const int* bhi, int* lo, int* hi) {
    for (int d = 0; d < 3; ++d) {
        lo[d] = std::max(alo[d], blo[d]);
        hi[d] = std::min(ahi[d], bhi[d]);
        if (lo[d] > hi[d]) return false;
    }
    return true;
}

long long region_cells(const int* lo, const int* hi) {
    return (long long)(hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1);
}

// Exchange tags: ghost cells of box b inside the (periodically extended) domain
// that lie in the valid region of box s (s may equal b for periodic images).
static void build_exchange(ocfd_level* L, std::vector<ExTag>& tags) {
    const ocfd_box& dom = L->desc.domain;
    int period[3];
    for (int d = 0; d < 3; ++d) period[d] = dom.hi[d] - dom.lo[d] + 1;
    const int nb = (int)L->boxes.size();
    for (int b = 0; b < nb; ++b) {
        const ocfd_box& B = L->boxes[b];
        int glo[3], ghi[3];
        const int nf = box_nfill(L, b);
        for (int d = 0; d < 3; ++d) { glo[d] = B.lo[d] - nf; ghi[d] = B.hi[d] + nf; }
        for (int sx = -1; sx <= 1; ++sx)
            for (int sy = -1; sy <= 1; ++sy)
                for (int sz = -1; sz <= 1; ++sz) {
                    const int sh[3] = {sx, sy, sz};
                    bool ok = true;
                    for (int d = 0; d < 3; ++d)
                        if (sh[d] != 0 && L->desc.lo_bc[d] != OCFD_BC_INTERIOR) ok = false;
                    if (!ok) continue;
                    for (int s = 0; s < nb; ++s) {
                        const ocfd_box& Sb = L->boxes[s];
                        // image of Sb shifted by sh * period
                        int ilo[3], ihi[3];
                        for (int d = 0; d < 3; ++d) {
                            ilo[d] = Sb.lo[d] + sh[d] * period[d];
                            ihi[d] = Sb.hi[d] + sh[d] * period[d];
                        }
                        int lo[3], hi[3];
                        if (!intersect(glo, ghi, ilo, ihi, lo, hi)) continue;
                        if (s == b && sx == 0 && sy == 0 && sz == 0) continue;  // own valid cells
                        // split the intersection into the parts outside box b's valid region:
                        // the region minus B, as up to 6 slabs
                        int rlo[3] = {lo[0], lo[1], lo[2]}, rhi[3] = {hi[0], hi[1], hi[2]};
                        for (int d = 0; d < 3; ++d) {
                            if (rlo[d] < B.lo[d]) {
                                ExTag t{};
                                t.dst = b; t.src = s;
                                for (int e = 0; e < 3; ++e) { t.lo[e] = rlo[e]; t.hi[e] = rhi[e]; t.shift[e] = -sh[e] * period[e]; }
                                t.hi[d] = std::min(rhi[d], B.lo[d] - 1);
                                tags.push_back(t);
                                rlo[d] = B.lo[d];
                            }
                            if (rhi[d] > B.hi[d]) {
                                ExTag t{};
                                t.dst = b; t.src = s;
                                for (int e = 0; e < 3; ++e) { t.lo[e] = rlo[e]; t.hi[e] = rhi[e]; t.shift[e] = -sh[e] * period[e]; }
                                t.lo[d] = std::max(rlo[d], B.hi[d] + 1);
                                tags.push_back(t);
                                rhi[d] = B.hi[d];
                            }
                            if (rlo[d] > rhi[d]) break;
                        }
                    }
                }
    }
}

// Physical-boundary tags of pass d for every box whose grown region leaves the domain in d.
static void build_physbc(ocfd_level* L, int d, std::vector<BcTag>& tags) {
    const ocfd_box& dom = L->desc.domain;
    if (L->desc.lo_bc[d] == OCFD_BC_INTERIOR) return;  // periodic: exchange fills it
    for (int b = 0; b < (int)L->boxes.size(); ++b) {
        const ocfd_box& B = L->boxes[b];
        for (int side = 0; side < 2; ++side) {
            BcTag t{};
            t.box = b;
            t.side = side;
            for (int e = 0; e < 3; ++e) {
                t.lo[e] = B.lo[e] - box_nfill(L, b);
                t.hi[e] = B.hi[e] + box_nfill(L, b);
                if (e > d && L->desc.lo_bc[e] != OCFD_BC_INTERIOR) {
                    t.lo[e] = std::max(t.lo[e], dom.lo[e]);
                    t.hi[e] = std::min(t.hi[e], dom.hi[e]);
                }
            }
            if (side == 0) t.hi[d] = std::min(t.hi[d], dom.lo[d] - 1);
            else t.lo[d] = std::max(t.lo[d], dom.hi[d] + 1);
            bool empty = false;
            for (int e = 0; e < 3; ++e) empty = empty || t.lo[e] > t.hi[e];
            if (!empty) tags.push_back(t);
        }
    }
}

int box_nfill(const ocfd_level* L, int b) {
    const int c = eb_box_class(L, b);
    return c == OCFD_BOX_REGULAR ? NFILL : (c == OCFD_BOX_CUT ? 2 : 1);
}

ocfd_status rebuild_fill_tags(ocfd_level* L) {
    DevPool* pool = L->pool;
    dev_free(L->d_ex, pool);
    dev_free(L->d_ex_start, pool);
    dev_free(L->d_ex_chunk, pool);
    L->d_ex = nullptr;
    L->d_ex_start = nullptr;
    L->d_ex_chunk = nullptr;
    std::vector<ExTag> ex;
    build_exchange(L, ex);
    L->nex = (int)ex.size();
    ocfd_status s = upload_tags(ex, &L->d_ex, &L->d_ex_start, &L->ex_total, pool, &L->d_ex_chunk);
    for (int d = 0; d < 3 && s == OCFD_OK; ++d) {
        dev_free(L->d_bc[d], pool);
        dev_free(L->d_bc_start[d], pool);
        dev_free(L->d_bc_chunk[d], pool);
        L->d_bc[d] = nullptr;
        L->d_bc_start[d] = nullptr;
        L->d_bc_chunk[d] = nullptr;
        std::vector<BcTag> bt;
        build_physbc(L, d, bt);
        L->nbc[d] = (int)bt.size();
        s = upload_tags(bt, &L->d_bc[d], &L->d_bc_start[d], &L->bc_total[d], pool, &L->d_bc_chunk[d]);
    }
    return s;
}

ocfd_status fill_exchange(ocfd_level* L, double* U, cudaStream_t st) {
    if (L->ex_total > 0)
        k_exchange<<<grid_for(L->ex_total, 256, L->ctx->num_sms), 256, 0, st>>>(
            L->d_ex, L->d_ex_start, L->d_ex_chunk, L->nex, L->ex_total, L->d_fabs, U, L->ncomp);
    return check_launch("level exchange");
}

ocfd_status fill_physbc(ocfd_level* L, double* U, double tfrac, cudaStream_t st, bool all) {
    const int sms = L->ctx->num_sms;
    if (L->bc_total[0] > 0)
        k_physbc<0><<<grid_for(L->bc_total[0], 256, sms), 256, 0, st>>>(
            L->d_bc[0], L->d_bc_start[0], L->d_bc_chunk[0], L->nbc[0], L->bc_total[0], L->d_fabs, U, L->ncomp,
            L->bcinfo, L->d_step, tfrac);
    if (L->bc_total[1] > 0)
        k_physbc<1><<<grid_for(L->bc_total[1], 256, sms), 256, 0, st>>>(
            L->d_bc[1], L->d_bc_start[1], L->d_bc_chunk[1], L->nbc[1], L->bc_total[1], L->d_fabs, U, L->ncomp,
            L->bcinfo, L->d_step, tfrac);
    if (L->bc_total[2] > 0 && (all || !L->zvirt))
        k_physbc<2><<<grid_for(L->bc_total[2], 256, sms), 256, 0, st>>>(
            L->d_bc[2], L->d_bc_start[2], L->d_bc_chunk[2], L->nbc[2], L->bc_total[2], L->d_fabs, U, L->ncomp,
            L->bcinfo, L->d_step, tfrac);
    return check_launch("level physical BC");
}

ocfd_status fill_ghosts(ocfd_level* L, double* U, double tfrac, cudaStream_t st, bool all) {
    ocfd_status s = fill_exchange(L, U, st);
    if (s != OCFD_OK) return s;
    return fill_physbc(L, U, tfrac, st, all);
}

ocfd_status launch_estdt(ocfd_level* L, cudaStream_t st) {
    const int sms = L->ctx->num_sms;
    k_reset_cfl<<<1, 1, 0, st>>>(L->d_step);
    k_estdt<<<grid_for(L->ncells, 256, sms), 256, 0, st>>>(
        L->d_fabs, L->d_cell_start, (int)L->boxes.size(), L->ncells, L->buf[0], L->ctx->parm,
        L->desc.dx[0], L->desc.dx[1], L->desc.dx[2], &L->d_step->cfl_min);
    return check_launch("level estdt");
}

ocfd_status launch_stage(ocfd_level* L, int s, unsigned flags, cudaStream_t st) {
    const bool visc = flags & OCFD_VISC;
    const bool f32 = flags & OCFD_FLUX_FP32;
    DevParm P = L->ctx->parm;
    P.grav = (flags & OCFD_GRAVITY) ? kGravity : 0.0;  // regular boxes only, as the reference
    ocfd_status r = OCFD_OK;
    if (flags & OCFD_PER_BOX) {
        // one launch per regular box (its tiles), then the cut boxes one by one
        for (int b = 0; b < L->nreg && r == OCFD_OK; ++b)
            r = f32 ? launch_rhs_regular_f32(L->tile, visc, nullptr, nullptr, 1, L->h_stage[s][b], L->h_ntiles[b],
                                             P, st)
                    : launch_rhs_regular(L->tile, visc, nullptr, nullptr, 1, L->h_stage[s][b], L->h_ntiles[b],
                                         P, st);
    } else if (L->ntiles > 0) {
        RegBoxArgs dummy{};
        r = f32 ? launch_rhs_regular_f32(L->tile, visc, L->d_stage[s], L->d_tile_start, L->nreg, dummy, L->ntiles,
                                         P, st, L->sched, L->d_queue)
                : launch_rhs_regular(L->tile, visc, L->d_stage[s], L->d_tile_start, L->nreg, dummy, L->ntiles,
                                     P, st, L->sched, L->d_queue);
    }
    if (r == OCFD_OK) r = eb_launch_stage(L, s, flags, st);
    return r;
}

ocfd_status level_autotune(ocfd_level* L, unsigned flags, int reps, cudaStream_t st) {
    if (L->nreg == 0 || reps <= 0) return OCFD_OK;
    // the stage tables are rebuilt below: no launch may still read them
    if (cudaDeviceSynchronize() != cudaSuccess) return check_launch("level autotune");
    const bool visc = flags & OCFD_VISC, f32 = flags & OCFD_FLUX_FP32;
    const StageRoles roles = L->roles ? *L->roles : StageRoles{};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    int bt = L->tile, bs = L->sched;
    ocfd_status s = OCFD_OK;
    for (int t = 0; t < kNumRegularTiles && s == OCFD_OK; ++t) {
        if (!regular_tile_fits(t, visc)) continue;
        if (kRegularTiles[t].staged && (!f32 || visc)) continue;  // the pencil kernel again
        L->tile = t;
        s = build_stage_tables(L, roles);
        for (int sc = 0; sc < NUM_SCHED && s == OCFD_OK; ++sc) {
            L->sched = sc;
            RegBoxArgs dummy{};
            auto go = [&]() {
                return f32 ? launch_rhs_regular_f32(L->tile, visc, L->d_stage[STAGE_PROBE], L->d_tile_start, L->nreg, dummy,
                                                    L->ntiles, L->ctx->parm, st, L->sched, L->d_queue)
                           : launch_rhs_regular(L->tile, visc, L->d_stage[STAGE_PROBE], L->d_tile_start, L->nreg, dummy,
                                                L->ntiles, L->ctx->parm, st, L->sched, L->d_queue);
            };
            s = go();  // warm-up
            cudaEventRecord(e0, st);
            for (int r = 0; r < reps && s == OCFD_OK; ++r) s = go();
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (s == OCFD_OK && ms < best) {
                best = ms;
                bt = t;
                bs = sc;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s != OCFD_OK) return s;
    L->tile = bt;
    L->sched = bs;
    s = build_stage_tables(L, roles);
    if (L->graph) {
        cudaGraphExecDestroy(L->graph);
        L->graph = nullptr;
    }
    if (s == OCFD_OK && cudaStreamSynchronize(st) != cudaSuccess) s = check_launch("level autotune");
    return s;
}

int stage_launches(const ocfd_level* L, unsigned flags) {
    return ((flags & OCFD_PER_BOX) ? L->nreg : (L->ntiles > 0 ? 1 : 0)) + eb_launches_per_stage(L, flags);
}

static ocfd_status record_step(ocfd_level* L, unsigned flags, cudaStream_t st) {
    k_step_begin<<<1, 1, 0, st>>>(L->d_step);
    const RkScheme& R = rk_scheme(L->rk_order);
    for (int s = 0; s < R.nst; ++s) {
        ocfd_status r = fill_ghosts(L, L->buf[R.src[s]], R.tfrac[s], st);
        if (r != OCFD_OK) return r;
        r = launch_stage(L, s, flags, st);
        if (r != OCFD_OK) return r;
    }
    if (R.copy_out && cudaMemcpyAsync(L->buf[0], L->buf[1], sizeof(double) * L->elems, cudaMemcpyDeviceToDevice,
                                      st) != cudaSuccess)
        return check_launch("level step: B -> A");
    k_step_end<<<1, 1, 0, st>>>(L->d_step);
    return check_launch("level step");
}

static ocfd_array4 fab_array(const ocfd_level* L, int b, int i) {
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

const RkScheme& rk_scheme(int order) {
    // SSP-RK3 in Shu-Osher form (AmrLevel::RK(3, ...), Source/Advance.cpp:141-148);
    // AMReX registers the stage fluxes with the RK3 weights 1/6, 1/6, 2/3
    static const RkScheme rk3{3, 3, {0, 1, 2}, {1, 2, RK_OUT}, {0.0, 0.75, 1.0 / 3.0}, {1.0, 0.25, 2.0 / 3.0},
                              {0.0, 1.0, 0.5}, {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0}, false};
    // Heun, Source/Advance.cpp:123-138: U* = U^n + dt L(U^n) (ghosts at t), then
    // U^{n+1} = U^n / 2 + (U* + dt L(U*)) / 2 (ghosts at t + dt); each stage's
    // fluxes are registered with 0.5 dt (compute_dSdt(..., 0.5*dt, ...))
    static const RkScheme rk2{2, 2, {0, 1, 0}, {1, RK_OUT, 0}, {0.0, 0.5, 0.0}, {1.0, 0.5, 0.0},
                              {0.0, 1.0, 0.0}, {0.5, 0.5, 0.0}, false};
    // forward Euler, Source/Advance.cpp:117-122: U^{n+1} = U^n + dt L(U^n)
    static const RkScheme rk1{1, 1, {0, 0, 0}, {1, 0, 0}, {0.0, 0.0, 0.0}, {1.0, 0.0, 0.0},
                              {0.0, 0.0, 0.0}, {1.0, 0.0, 0.0}, true};
    return order == 1 ? rk1 : (order == 2 ? rk2 : rk3);
}

StageSlot stage_slot(int order, const StageRoles& roles, int k) {
    StageSlot z{};
    if (k == STAGE_PROBE) {
        const RkScheme& R = rk_scheme(3);
        return StageSlot{true, R.src[1], R.out[1], R.a[1], R.b[1], R.w[1], false};
    }
    const RkScheme& R = rk_scheme(order);
    if (k < 0 || k >= R.nst) return z;
    const int out = R.out[k] == RK_OUT ? roles.out3 : R.out[k];
    return StageSlot{true, R.src[k], out, R.a[k], R.b[k], R.w[k], k == R.nst - 1 && roles.cfl};
}

// Stage tables, one per slot (stage_slot): for SSP-RK3 stage 1 A -> B, stage 2
// (A, B) -> C, stage 3 (A, C) -> A (or D)
ocfd_status build_stage_tables(ocfd_level* L, const StageRoles& roles) {
    if (L->roles != &roles) {
        delete L->roles;
        L->roles = new StageRoles(roles);
    }
    const ocfd_level_desc* desc = &L->desc;
    const double dxinv[3] = {1.0 / desc->dx[0], 1.0 / desc->dx[1], 1.0 / desc->dx[2]};
    std::vector<int> tile_start;
    int nt = 0;
    std::vector<RegBoxArgs> st[NUM_STAGE_SLOTS];
    StageSlot slot[NUM_STAGE_SLOTS];
    for (int k = 0; k < NUM_STAGE_SLOTS; ++k) slot[k] = stage_slot(L->rk_order, roles, k);
    for (size_t b = 0; b < L->boxes.size(); ++b) {
        if (!eb_box_regular(L, (int)b)) continue;  // cut / covered: eb_level.cu
        ocfd_array4 a[4];
        for (int i = 0; i < L->nbuf; ++i) a[i] = fab_array(L, (int)b, i);
        for (int k = 0; k < NUM_STAGE_SLOTS; ++k) {
            if (!slot[k].used) continue;
            RegBoxArgs r{};
            fill_regular_args(r, &a[slot[k].src], nullptr, nullptr, L->boxes[b], dxinv, L->tile);
            r.mode = RHS_FUSED_STAGE;
            r.U0 = view_of<const double>(&a[0]);
            r.Uout = view_of<double>(&a[slot[k].out]);
            r.rk_a = slot[k].a;
            r.rk_b = slot[k].b;
            r.dt_ptr = &L->d_step->dt;
            r.zvirt = L->zvirt ? 1 : 0;
            r.zdom[0] = desc->domain.lo[2];
            r.zdom[1] = desc->domain.hi[2];
            for (int sd = 0; sd < 2; ++sd) {
                r.zmirror[sd] = L->zmirror[sd];
                r.zsign[sd] = L->zsign[sd];
            }
            r.cfl_min = slot[k].cfl ? &L->d_step->cfl_min : nullptr;
            for (int d = 0; d < 3; ++d) {
                r.dx[d] = desc->dx[d];
                r.dx_f[d] = (float)desc->dx[d];
            }
            if (!roles.flux_bits.empty() && roles.flux_bits[b]) {
                r.has_flux = roles.flux_bits[b];
                r.flux_w = slot[k].w;
                if (r.has_flux & FLUX_ACC_ALL)
                    for (int d = 0; d < 3; ++d) r.flux[d] = roles.creg[3 * b + d];
                if (r.has_flux & FLUX_ACC_PLANES)
                    for (int d = 0; d < 3; ++d)
                        for (int sd = 0; sd < 2; ++sd) r.fplane[d][sd] = roles.fplane[6 * b + 2 * d + sd];
            }
            st[k].push_back(r);
            if (k == 0) {
                tile_start.push_back(nt);
                nt += r.ntile[0] * r.ntile[1] * r.ntile[2];
            }
        }
    }
    L->ntiles = nt;
    L->nreg = (int)tile_start.size();
    L->h_ntiles.clear();
    for (int b = 0; b < L->nreg; ++b) L->h_ntiles.push_back((b + 1 < L->nreg ? tile_start[b + 1] : nt) - tile_start[b]);
    for (int k = 0; k < NUM_STAGE_SLOTS; ++k) L->h_stage[k] = st[k];
    ocfd_status s = OCFD_OK;
    for (int k = 0; k < NUM_STAGE_SLOTS && s == OCFD_OK; ++k) {
        dev_free(L->d_stage[k], L->pool);
        L->d_stage[k] = nullptr;
        s = upload(&L->d_stage[k], st[k], L->pool);
    }
    dev_free(L->d_tile_start, L->pool);
    L->d_tile_start = nullptr;
    if (s == OCFD_OK) s = upload(&L->d_tile_start, tile_start, L->pool);
    if (s == OCFD_OK) s = eb_build_stage_tables(L, roles);
    return s;
}

// The boxes of one level are disjoint (an AMReX BoxArray of a level): sweep
// over the boxes in order of lo.x, testing each against those that start
// before it ends in x.
static bool boxes_disjoint(const std::vector<ocfd_box>& b) {
    std::vector<int> ord(b.size());
    for (size_t i = 0; i < b.size(); ++i) ord[i] = (int)i;
    std::sort(ord.begin(), ord.end(), [&](int u, int v) { return b[u].lo[0] < b[v].lo[0]; });
    for (size_t a = 0; a < ord.size(); ++a) {
        const ocfd_box& A = b[ord[a]];
        for (size_t c = a + 1; c < ord.size() && b[ord[c]].lo[0] <= A.hi[0]; ++c) {
            const ocfd_box& C = b[ord[c]];
            if (C.lo[1] <= A.hi[1] && A.lo[1] <= C.hi[1] && C.lo[2] <= A.hi[2] && A.lo[2] <= C.hi[2])
                return false;
        }
    }
    return true;
}

// Everything of a level but its stage tables: FABs, state buffers, exchange and
// physical-BC tags, RHS tile choice, step state.
ocfd_status level_alloc(ocfd_context* ctx, const ocfd_level_desc* desc, int nbuf, ocfd_level** out,
                        DevPool* pool, int ncomp) {
    if (!ctx || !desc || !out || desc->nbox <= 0 || !desc->boxes || nbuf < 3 || nbuf > 4)
        return fail(OCFD_BAD_ARG, "ocfd_level_create: bad arguments");
    *out = nullptr;
    for (int d = 0; d < 3; ++d) {
        if ((desc->lo_bc[d] == OCFD_BC_INTERIOR) != (desc->hi_bc[d] == OCFD_BC_INTERIOR))
            return fail(OCFD_BAD_ARG, "ocfd_level_create: periodic directions need interior BC on both sides");
        if (desc->lo_bc[d] < 0 || desc->lo_bc[d] > 5 || desc->hi_bc[d] < 0 || desc->hi_bc[d] > 5)
            return fail(OCFD_BAD_ARG, "ocfd_level_create: BC codes are 0..5");
        if (!(desc->dx[d] > 0)) return fail(OCFD_BAD_ARG, "ocfd_level_create: dx must be positive");
    }
    ocfd_level* L = new ocfd_level();
    L->ctx = ctx;
    L->desc = *desc;
    L->nbuf = nbuf;
    L->pool = pool;
    L->ncomp = ncomp;
    L->boxes.assign(desc->boxes, desc->boxes + desc->nbox);
    L->desc.boxes = nullptr;
    long long off = 0;
    std::vector<long long> cell_start;
    for (const ocfd_box& B : L->boxes) {
        FabGeom f{};
        for (int d = 0; d < 3; ++d) {
            if (B.hi[d] < B.lo[d] || B.lo[d] < desc->domain.lo[d] || B.hi[d] > desc->domain.hi[d]) {
                delete L;
                return fail(OCFD_BAD_ARG, "ocfd_level_create: box outside the domain or empty");
            }
            f.lo[d] = B.lo[d];
            f.hi[d] = B.hi[d];
            f.g[d] = B.hi[d] - B.lo[d] + 1 + 2 * NGR;
        }
        f.ns = (long long)f.g[0] * f.g[1] * f.g[2];
        f.off = off;
        off += f.ns * L->ncomp;
        cell_start.push_back(L->ncells);
        L->ncells += region_cells(f.lo, f.hi);
        L->fabs.push_back(f);
    }
    if (!boxes_disjoint(L->boxes)) {
        delete L;
        return fail(OCFD_BAD_ARG, "ocfd_level_create: boxes overlap");
    }
    L->elems = off;
    for (int i = 0; i < nbuf; ++i) {
        L->buf[i] = static_cast<double*>(dev_alloc(sizeof(double) * L->elems, pool));
        if (!L->buf[i]) {
            ocfd_level_destroy(L);
            return fail(OCFD_OUT_OF_MEMORY, "ocfd_level_create: state buffers");
        }
        if (!pool) cudaMemset(L->buf[i], 0, sizeof(double) * L->elems);
    }
    ocfd_status s = upload(&L->d_fabs, L->fabs, pool);
    if (s == OCFD_OK) s = upload(&L->d_cell_start, cell_start, pool);
    std::vector<ExTag> ex;
    build_exchange(L, ex);
    L->nex = (int)ex.size();
    if (s == OCFD_OK) s = upload_tags(ex, &L->d_ex, &L->d_ex_start, &L->ex_total, pool, &L->d_ex_chunk);
    for (int d = 0; d < 3 && s == OCFD_OK; ++d) {
        std::vector<BcTag> bt;
        build_physbc(L, d, bt);
        L->nbc[d] = (int)bt.size();
        s = upload_tags(bt, &L->d_bc[d], &L->d_bc_start[d], &L->bc_total[d], pool, &L->d_bc_chunk[d]);
    }
    for (int d = 0; d < 3; ++d) {
        L->bcinfo.lo_bc[d] = desc->lo_bc[d];
        L->bcinfo.hi_bc[d] = desc->hi_bc[d];
        L->bcinfo.dom_lo[d] = desc->domain.lo[d];
        L->bcinfo.dom_hi[d] = desc->domain.hi[d];
        L->bcinfo.dx[d] = desc->dx[d];
        L->bcinfo.prob_lo[d] = desc->prob_lo[d];
    }
    L->bcinfo.bc_case = desc->bc_case;
    // outflow (foextrap), symmetry / slip wall (reflect, w odd) and no-slip wall
    // (reflect, u v w odd) take z ghosts from inside the domain, Source/Setup.cpp:22-35;
    // no case functor writes z faces
    {
        const int zb[2] = {desc->lo_bc[2], desc->hi_bc[2]};
        bool simple = true;
        for (int sd = 0; sd < 2; ++sd) {
            simple = simple && zb[sd] >= 2 && zb[sd] <= 5;
            L->zmirror[sd] = zb[sd] >= 3 ? 1 : 0;
            L->zsign[sd] = zb[sd] == 5 ? 7 : (zb[sd] >= 3 ? 4 : 0);
        }
        L->zvirt = simple;
        L->zvirt_allowed = simple;
    }
    std::memcpy(L->bcinfo.params, desc->case_params, sizeof(L->bcinfo.params));
    // RHS tile: the shape with the least padded work summed over the boxes
    if (desc->tile >= 0 && desc->tile < kNumRegularTiles) {
        L->tile = desc->tile;
    } else {
        double best = 1e300;
        for (int t = 0; t < kNumRegularTiles; ++t) {
            if (!regular_tile_fits(t, true) || kRegularTiles[t].staged) continue;
            const TileShape& ts = kRegularTiles[t];
            double cost = 0;
            for (const ocfd_box& B : L->boxes) {
                const int n[3] = {B.hi[0] - B.lo[0] + 1, B.hi[1] - B.lo[1] + 1, B.hi[2] - B.lo[2] + 1};
                long long tiles = (long long)((n[0] + ts.x - 1) / ts.x) * ((n[1] + ts.y - 1) / ts.y) * ((n[2] + ts.z - 1) / ts.z);
                cost += tiles * ((double)ts.x * ts.y * ts.z * 3.0 + 6.0 * ((double)ts.y * ts.z + (double)ts.x * ts.z + (double)ts.x * ts.y));
            }
            if (cost < best * 0.999) { best = cost; L->tile = t; }
        }
    }
    if (s == OCFD_OK) {
        L->d_step = static_cast<StepState*>(dev_alloc(sizeof(StepState), pool));
        L->d_queue = static_cast<unsigned*>(dev_alloc(2 * sizeof(unsigned), pool));
        if (!L->d_step || !L->d_queue) s = fail(OCFD_OUT_OF_MEMORY, "step state");
        else if (cudaMemset(L->d_queue, 0, 2 * sizeof(unsigned)) != cudaSuccess) s = check_launch("work queue");
    }
    if (s == OCFD_OK) {
        k_set_time<<<1, 1>>>(L->d_step, 0.0);
        k_set_stop<<<1, 1>>>(L->d_step, __builtin_huge_val());
        s = check_launch("ocfd_level_create");
    }
    if (s != OCFD_OK) {
        ocfd_level_destroy(L);
        return s;
    }
    *out = L;
    return OCFD_OK;
}

// Valid cells of every box <-> the dense list `valid` (box after box in box
// order, each (ncomp, nz, ny, nx), i fastest); to_fab = 1 writes the FABs.
__global__ void k_valid_copy(const FabGeom* __restrict__ fabs, const long long* __restrict__ cell_start, int nbox,
                             long long ncells, int ncomp, double* __restrict__ U, double* __restrict__ valid,
                             int to_fab) {
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < ncells;
         idx += (long long)gridDim.x * blockDim.x) {
        const int b = find_tag<FabGeom>(cell_start, nbox, idx);
        const FabGeom& f = fabs[b];
        const long long local = idx - cell_start[b];
        const int nx = f.hi[0] - f.lo[0] + 1, ny = f.hi[1] - f.lo[1] + 1;
        const long long nb = (long long)nx * ny * (f.hi[2] - f.lo[2] + 1);
        const int i = f.lo[0] + (int)(local % nx), j = f.lo[1] + (int)((local / nx) % ny),
                  k = f.lo[2] + (int)(local / ((long long)nx * ny));
        const long long g = fab_index(f, i, j, k);
        double* v = valid + cell_start[b] * ncomp + local;
        if (to_fab)
            for (int n = 0; n < ncomp; ++n) U[g + n * f.ns] = v[n * nb];
        else
            for (int n = 0; n < ncomp; ++n) v[n * nb] = U[g + n * f.ns];
    }
}

static bool is_device_pointer(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

static ocfd_status valid_staging(ocfd_level* L) {
    if (L->d_valid) return OCFD_OK;
    L->d_valid = static_cast<double*>(dev_alloc(sizeof(double) * std::max<long long>(1, L->ncells * L->ncomp), L->pool));
    return L->d_valid ? OCFD_OK : fail(OCFD_OUT_OF_MEMORY, "level valid-cell staging");
}

ocfd_status level_copy_valid(ocfd_level* L, double* buf, bool in, cudaStream_t st) {
    const bool dev = is_device_pointer(buf);
    if (!dev) {
        ocfd_status s = valid_staging(L);
        if (s != OCFD_OK) return s;
    }
    const size_t bytes = sizeof(double) * L->ncells * L->ncomp;
    double* list = dev ? buf : L->d_valid;
    if (in && !dev && cudaMemcpyAsync(L->d_valid, buf, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return check_launch("valid-cell copy in");
    if (L->ncells > 0)
        k_valid_copy<<<grid_for(L->ncells, 256, L->ctx->num_sms), 256, 0, st>>>(
            L->d_fabs, L->d_cell_start, (int)L->boxes.size(), L->ncells, L->ncomp, L->buf[0], list, in ? 1 : 0);
    ocfd_status s = check_launch("valid-cell copy");
    if (s == OCFD_OK && !in && !dev && cudaMemcpyAsync(buf, L->d_valid, bytes, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        s = check_launch("valid-cell copy out");
    return s;
}

}  // namespace ocfd

extern "C" {

ocfd_status ocfd_level_create(ocfd_context* ctx, const ocfd_level_desc* desc, ocfd_level** out) {
    ocfd_level* L = nullptr;
    ocfd_status s = level_alloc(ctx, desc, 3, &L);
    if (s != OCFD_OK) return s;
    s = build_stage_tables(L, StageRoles{});
    if (s == OCFD_OK && cudaDeviceSynchronize() != cudaSuccess) s = fail(OCFD_LAUNCH_FAIL, "level setup");
    if (s != OCFD_OK) {
        ocfd_level_destroy(L);
        return s;
    }
    *out = L;
    return OCFD_OK;
}

ocfd_status ocfd_level_destroy(ocfd_level* L) {
    if (!L) return OCFD_OK;
    if (L->graph) cudaGraphExecDestroy(L->graph);
    eb_free(L);
    delete L->roles;
    DevPool* pool = L->pool;
    for (int i = 0; i < 4; ++i) dev_free(L->buf[i], pool);
    for (int i = 0; i < NUM_STAGE_SLOTS; ++i) dev_free(L->d_stage[i], pool);
    dev_free(L->d_valid, pool);
    for (int i = 0; i < 3; ++i) {
        dev_free(L->d_bc[i], pool);
        dev_free(L->d_bc_start[i], pool);
        dev_free(L->d_bc_chunk[i], pool);
    }
    dev_free(L->d_fabs, pool);
    dev_free(L->d_cell_start, pool);
    dev_free(L->d_ex, pool);
    dev_free(L->d_ex_start, pool);
    dev_free(L->d_ex_chunk, pool);
    dev_free(L->d_tile_start, pool);
    dev_free(L->d_step, pool);
    dev_free(L->d_queue, pool);
    delete L;
    return OCFD_OK;
}

ocfd_status ocfd_level_state(ocfd_level* L, int ibox, ocfd_array4* out) {
    if (!L || !out || ibox < 0 || ibox >= (int)L->boxes.size()) return fail(OCFD_BAD_ARG, "ocfd_level_state");
    const FabGeom& f = L->fabs[ibox];
    out->p = L->buf[0] + f.off;
    out->jstride = f.g[0];
    out->kstride = (long long)f.g[0] * f.g[1];
    out->nstride = f.ns;
    for (int d = 0; d < 3; ++d) {
        out->begin[d] = f.lo[d] - NGR;
        out->end[d] = f.hi[d] + NGR + 1;
    }
    out->ncomp = L->ncomp;
    return OCFD_OK;
}

size_t ocfd_level_state_elems(const ocfd_level* L) { return L ? (size_t)L->elems : 0; }

ocfd_status ocfd_level_set_schedule(ocfd_level* L, int32_t tile, int32_t sched) {
    if (!L || sched < 0 || sched >= NUM_SCHED || tile < -1 || tile >= kNumRegularTiles ||
        (tile >= 0 && !regular_tile_fits(tile, false)))
        return fail(OCFD_BAD_ARG, "ocfd_level_set_schedule");
    L->sched = sched;
    ocfd_status s = OCFD_OK;
    if (tile >= 0 && tile != L->tile) {
        // the stage tables are rebuilt: no launch may still read them
        if (cudaDeviceSynchronize() != cudaSuccess) return check_launch("ocfd_level_set_schedule");
        L->tile = tile;
        const StageRoles roles = L->roles ? *L->roles : StageRoles{};
        s = build_stage_tables(L, roles);
    }
    if (L->graph) {
        cudaGraphExecDestroy(L->graph);
        L->graph = nullptr;
    }
    return s;
}

ocfd_status ocfd_level_set_time_integration(ocfd_level* L, int32_t order) {
    if (!L || order < 1 || order > 3) return fail(OCFD_BAD_ARG, "ocfd_level_set_time_integration: order is 1, 2 or 3");
    if (L->ncomp != 5) return fail(OCFD_BAD_ARG, "ocfd_level_set_time_integration: a reacting level sets its order at creation");
    if (L->pool) return fail(OCFD_BAD_ARG, "ocfd_level_set_time_integration: a hierarchy's level follows ocfd_amr_set_time_integration");
    if (order == L->rk_order) return OCFD_OK;
    if (cudaDeviceSynchronize() != cudaSuccess) return check_launch("ocfd_level_set_time_integration");
    L->rk_order = order;
    const StageRoles roles = L->roles ? *L->roles : StageRoles{};
    ocfd_status s = build_stage_tables(L, roles);
    if (L->graph) {
        cudaGraphExecDestroy(L->graph);
        L->graph = nullptr;
    }
    return s;
}

ocfd_status ocfd_level_autotune(ocfd_level* L, unsigned flags, int reps, int32_t* tile, int32_t* sched,
                                void* stream) {
    if (!L || reps <= 0) return fail(OCFD_BAD_ARG, "ocfd_level_autotune");
    ocfd_status s = level_autotune(L, flags, reps, static_cast<cudaStream_t>(stream));
    if (tile) *tile = L->tile;
    if (sched) *sched = L->sched;
    return s;
}

ocfd_status ocfd_level_copy_in(ocfd_level* L, const double* buf, void* stream) {
    if (!L || !buf) return fail(OCFD_BAD_ARG, "ocfd_level_copy_in");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemcpyAsync(L->buf[0], buf, sizeof(double) * L->elems, cudaMemcpyDefault, st) != cudaSuccess)
        return check_launch("ocfd_level_copy_in");
    L->need_estdt = true;
    k_set_time<<<1, 1, 0, st>>>(L->d_step, 0.0);
    return check_launch("ocfd_level_copy_in");
}

ocfd_status ocfd_level_copy_valid_in(ocfd_level* L, const double* buf, void* stream) {
    if (!L || !buf) return fail(OCFD_BAD_ARG, "ocfd_level_copy_valid_in");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    ocfd_status s = level_copy_valid(L, const_cast<double*>(buf), true, st);
    if (s != OCFD_OK) return s;
    L->need_estdt = true;
    k_set_time<<<1, 1, 0, st>>>(L->d_step, 0.0);
    return check_launch("ocfd_level_copy_valid_in");
}

ocfd_status ocfd_level_copy_valid_out(ocfd_level* L, double* buf, void* stream) {
    if (!L || !buf) return fail(OCFD_BAD_ARG, "ocfd_level_copy_valid_out");
    return level_copy_valid(L, buf, false, static_cast<cudaStream_t>(stream));
}

int64_t ocfd_level_valid_elems(const ocfd_level* L) { return L ? (int64_t)L->ncells * L->ncomp : 0; }

ocfd_status ocfd_level_copy_out(ocfd_level* L, double* buf, void* stream) {
    if (!L || !buf) return fail(OCFD_BAD_ARG, "ocfd_level_copy_out");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemcpyAsync(buf, L->buf[0], sizeof(double) * L->elems, cudaMemcpyDefault, st) != cudaSuccess)
        return check_launch("ocfd_level_copy_out");
    return OCFD_OK;
}

ocfd_status ocfd_level_fill_ghosts(ocfd_level* L, double time, void* stream) {
    if (!L) return fail(OCFD_BAD_ARG, "ocfd_level_fill_ghosts");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_set_time<<<1, 1, 0, st>>>(L->d_step, time);
    ocfd_status s = fill_ghosts(L, L->buf[0], 0.0, st, true);
    L->need_estdt = true;
    return s;
}

ocfd_status ocfd_level_set_time(ocfd_level* L, double time, void* stream) {
    if (!L) return fail(OCFD_BAD_ARG, "ocfd_level_set_time");
    k_set_time<<<1, 1, 0, static_cast<cudaStream_t>(stream)>>>(L->d_step, time);
    L->need_estdt = true;
    return check_launch("ocfd_level_set_time");
}

ocfd_status ocfd_level_advance(ocfd_level* L, int nsteps, double cfl, unsigned flags, void* stream) {
    if (!L || nsteps < 0 || !(cfl > 0)) return fail(OCFD_BAD_ARG, "ocfd_level_advance");
    if (flags & ~(unsigned)(OCFD_VISC | OCFD_FLUX_FP32 | OCFD_PER_BOX | OCFD_GRAVITY))
        return fail(OCFD_BAD_ARG, "ocfd_level_advance: flags");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (nsteps == 0) return OCFD_OK;
    if (cudaMemcpyAsync(&L->d_step->cfl, &cfl, sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess)
        return check_launch("ocfd_level_advance");
    if (L->need_estdt) {
        ocfd_status s = launch_estdt(L, st);
        if (s != OCFD_OK) return s;
        L->need_estdt = false;
    }
    if (flags & OCFD_PER_BOX) {  // host-issued launches, step after step
        for (int i = 0; i < nsteps; ++i) {
            ocfd_status s = record_step(L, flags, st);
            if (s != OCFD_OK) return s;
        }
        return OCFD_OK;
    }
    if (!L->graph || L->graph_flags != flags) {
        if (L->graph) {
            cudaGraphExecDestroy(L->graph);
            L->graph = nullptr;
        }
        // capture on a private stream so the caller's stream may be the legacy default
        cudaStream_t cap;
        if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return check_launch("capture stream");
        cudaGraph_t g;
        if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaStreamDestroy(cap);
            return check_launch("begin capture");
        }
        ocfd_status s = record_step(L, flags, cap);
        cudaError_t e = cudaStreamEndCapture(cap, &g);
        cudaStreamDestroy(cap);
        if (s != OCFD_OK) return s;
        if (e != cudaSuccess) return fail(OCFD_LAUNCH_FAIL, std::string("end capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&L->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(OCFD_LAUNCH_FAIL, std::string("graph instantiate: ") + cudaGetErrorString(e));
        L->graph_flags = flags;
    }
    for (int i = 0; i < nsteps; ++i)
        if (cudaGraphLaunch(L->graph, st) != cudaSuccess) return check_launch("graph launch");
    return OCFD_OK;
}

ocfd_status ocfd_level_time(ocfd_level* L, double* time, double* last_dt, void* stream) {
    if (!L) return fail(OCFD_BAD_ARG, "ocfd_level_time");
    StepState h{};
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemcpyAsync(&h, L->d_step, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return check_launch("ocfd_level_time");
    if (time) *time = h.time;
    if (last_dt) *last_dt = h.dt_prev;
    return OCFD_OK;
}

int64_t ocfd_level_cells(const ocfd_level* L) { return L ? L->ncells : 0; }

ocfd_status ocfd_level_set_stop_time(ocfd_level* L, double stop_time, void* stream) {
    if (!L) return fail(OCFD_BAD_ARG, "ocfd_level_set_stop_time");
    k_set_stop<<<1, 1, 0, static_cast<cudaStream_t>(stream)>>>(L->d_step, stop_time);
    return check_launch("ocfd_level_set_stop_time");
}

int ocfd_level_launches_per_step(const ocfd_level* L, unsigned flags) {
    if (!L) return 0;
    (void)flags;
    int fill = (L->ex_total > 0) + (L->bc_total[0] > 0) + (L->bc_total[1] > 0) + (L->bc_total[2] > 0 && !L->zvirt);
    return 2 + rk_scheme(L->rk_order).nst * (fill + stage_launches(L, flags));
}

ocfd_status ocfd_level_profile_stage(ocfd_level* L, unsigned flags, int reps, double* ms, void* stream) {
    return ocfd_level_profile_part(L, flags, 0, reps, ms, nullptr, stream);
}

ocfd_status ocfd_level_profile_part(ocfd_level* L, unsigned flags, int part, int reps, double* ms, int64_t* cells,
                                    void* stream) {
    if (!L || reps <= 0 || !ms || part < 0 || part > 1) return fail(OCFD_BAD_ARG, "ocfd_level_profile_part");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cells) {
        long long n = 0;
        if (part == 0) {
            n = L->ncells;
        } else {
            for (const RegBoxArgs& a : L->h_stage[STAGE_PROBE])
                n += (long long)(a.hi[0] - a.lo[0] + 1) * (a.hi[1] - a.lo[1] + 1) * (a.hi[2] - a.lo[2] + 1);
        }
        *cells = n;
    }
    auto launch = [&]() {
        if (part == 0) return launch_stage(L, STAGE_PROBE, flags, st);
        // the regular boxes' tile kernel alone, as launch_stage issues it
        if (L->ntiles <= 0) return OCFD_OK;
        DevParm P = L->ctx->parm;
        P.grav = (flags & OCFD_GRAVITY) ? kGravity : 0.0;
        RegBoxArgs dummy{};
        const bool visc = flags & OCFD_VISC;
        return (flags & OCFD_FLUX_FP32)
                   ? launch_rhs_regular_f32(L->tile, visc, L->d_stage[STAGE_PROBE], L->d_tile_start, L->nreg, dummy,
                                            L->ntiles, P, st, L->sched, L->d_queue)
                   : launch_rhs_regular(L->tile, visc, L->d_stage[STAGE_PROBE], L->d_tile_start, L->nreg, dummy,
                                        L->ntiles, P, st, L->sched, L->d_queue);
    };
    ocfd_status s = launch();  // warm-up
    if (s != OCFD_OK) return s;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    for (int r = 0; r < reps && s == OCFD_OK; ++r) s = launch();
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = t / reps;
    return s;
}

}  // extern "C"
