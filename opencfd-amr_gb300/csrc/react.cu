// Reacting level: the multispecies flow of Source/CHEM with operator-split
// chemistry, on the device, one CUDA graph per step (EBR::advance, CHEM branch,
// Source/Advance.cpp:152-177, and EBR::post_timestep, Source/EBR.cpp:333-357):
//
//   chemistry half step : n substeps of dt / (2 n)   (EBR::chemical_advance)
//   flow step           : RK2 (Source/CHEM/FlowAdvance.cpp:95-122) or SSP-RK3,
//                         each stage = ghost fill of 5 + 9 components, the
//                         multispecies RHS chain per box, one combine kernel
//                         U_out = a U^n + b (U_s + dt L(U_s)) over the level
//   chemistry half step
//   species renormalisation
//
// State FABs hold 14 components: rho, rho u, rho v, rho w, rho E, then the 9
// partial densities (the Spec MultiFab of the reference) in the same FAB.
// Chemistry either runs per box, or (binned) as one launch over a list of all
// the level's cells ordered by a temperature key, so that the warps' Newton
// iterations for T(e) see similar states (the per-cell arithmetic is the same
// function, so results do not depend on the order).
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "chem_internal.h"
#include "eb_level.h"
#include "level.h"

namespace ocfd {

constexpr int NCOMP_REACT = 5 + NSP;
constexpr int NBIN = 32;

__global__ void k_react_combine(const FabGeom* __restrict__ fabs, const long long* __restrict__ start, int nbox,
                                long long total, double* out, const double* __restrict__ U0,
                                const double* __restrict__ S, const double* __restrict__ R, double a, double b,
                                const StepState* st) {
    const double dt = st->dt;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int bx = find_tag<FabGeom>(start, nbox, idx);
        const FabGeom& f = fabs[bx];
        int i, j, k;
        region_cell(f.lo, f.hi, idx - start[bx], i, j, k);
        const long long c = fab_index(f, i, j, k);
        for (int n = 0; n < NCOMP_REACT; ++n) {
            const long long q = c + n * f.ns;
            out[q] = a * U0[q] + b * (S[q] + dt * R[q]);
        }
    }
}

// temperature key: the linear estimate e / sum((a0 - 1) R / W_i rho_i) that
// starts the Newton iteration for T(e) (LiDryer.H:833-888), in 100 K bins
__global__ void k_react_keys(const FabGeom* __restrict__ fabs, const long long* __restrict__ start, int nbox,
                             long long total, const double* __restrict__ U, const double* __restrict__ a0w,
                             unsigned char* key, unsigned* count) {
    __shared__ unsigned hist[NBIN];
    for (int q = threadIdx.x; q < NBIN; q += blockDim.x) hist[q] = 0;
    __syncthreads();
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int bx = find_tag<FabGeom>(start, nbox, idx);
        const FabGeom& f = fabs[bx];
        int i, j, k;
        region_cell(f.lo, f.hi, idx - start[bx], i, j, k);
        const long long c = fab_index(f, i, j, k);
        const double rho = U[c];
        const double ke = 0.5 * (U[c + f.ns] * U[c + f.ns] + U[c + 2 * f.ns] * U[c + 2 * f.ns] +
                                 U[c + 3 * f.ns] * U[c + 3 * f.ns]) / rho;
        double As = 0.0;
        for (int n = 0; n < NSP; ++n) As += a0w[n] * U[c + (5 + n) * f.ns];
        const double T = (U[c + 4 * f.ns] - ke) / As;
        int b = (int)(T * 0.01);
        b = b < 0 ? 0 : (b >= NBIN ? NBIN - 1 : b);
        key[idx] = (unsigned char)b;
        atomicAdd(&hist[b], 1u);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < NBIN; q += blockDim.x)
        if (hist[q]) atomicAdd(&count[q], hist[q]);
}

__global__ void k_react_scan(unsigned* count) {
    unsigned acc = 0;
    for (int q = 0; q < NBIN; ++q) {
        const unsigned c = count[q];
        count[q] = acc;  // becomes the cursor of bin q
        acc += c;
    }
}

__global__ void k_react_scatter(const FabGeom* __restrict__ fabs, const long long* __restrict__ start, int nbox,
                                long long total, const unsigned char* __restrict__ key, unsigned* cursor,
                                long long* off, long long* stride) {
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int bx = find_tag<FabGeom>(start, nbox, idx);
        const FabGeom& f = fabs[bx];
        int i, j, k;
        region_cell(f.lo, f.hi, idx - start[bx], i, j, k);
        const unsigned pos = atomicAdd(&cursor[key[idx]], 1u);
        off[pos] = fab_index(f, i, j, k);
        stride[pos] = f.ns;
    }
}

__global__ void k_react_identity(const FabGeom* __restrict__ fabs, const long long* __restrict__ start, int nbox,
                                 long long total, long long* off, long long* stride) {
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int bx = find_tag<FabGeom>(start, nbox, idx);
        const FabGeom& f = fabs[bx];
        int i, j, k;
        region_cell(f.lo, f.hi, idx - start[bx], i, j, k);
        off[idx] = fab_index(f, i, j, k);
        stride[idx] = f.ns;
    }
}

__global__ void k_react_begin(StepState* st, double dt) {
    st->dt = dt;
}

__global__ void k_react_end(StepState* st) {
    st->time += st->dt;
    st->dt_prev = st->dt;
}

}  // namespace ocfd

struct ocfd_react {
    ocfd_context* ctx = nullptr;
    ocfd_react_desc desc{};
    ocfd_level* L = nullptr;     // 14-component FABs: A (U^n), B, C
    double* rhs = nullptr;       // L(U_s), same FAB layout
    double* scr = nullptr;       // multispecies RHS scratch of the largest box
    std::vector<ocfd::ChemBoxArgs> args[3];  // RHS chain of each box, per stage input buffer
    // embedded body: box classes (empty: every box regular) and the boxes the
    // chemistry visits (EBR::chemical_advance skips covered boxes,
    // Source/CHEM/ChemAdvance.cpp:20): their FAB table, cell prefix and cells
    std::vector<int> cls;
    ocfd::FabGeom* d_afabs = nullptr;
    long long* d_astart = nullptr;
    int nabox = 0;
    long long nactive = 0;
    // binned chemistry
    unsigned char* key = nullptr;
    unsigned* count = nullptr;
    long long* off = nullptr;
    long long* stride = nullptr;
    double* a0w = nullptr;
    // surrogate chemistry: network, guard, fallback list and counters
    ocfd_mlp* mlp = nullptr;
    ocfd_surrogate_guard guard{};
    long long* fb_off = nullptr;
    long long* fb_stride = nullptr;
    unsigned* fb_count = nullptr;
    unsigned long long* fb_total = nullptr;
    cudaGraphExec_t graph = nullptr;
    unsigned graph_flags = ~0u;
    int launches = 0;
};

namespace ocfd {

static ocfd_array4 fab_view(const ocfd_level* L, double* base, int b, int comp0, int ncomp) {
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

// One half step of chemistry (chem_substeps substeps of dt / 2 / chem_substeps).
// With `last` (the second half of a step) the last substep also renormalises
// the species of every cell it advances (Source/EBR.cpp:333-357, fused into its
// epilogue); returns in `renormed` whether it did (not in the surrogate form,
// whose cells finish in two kernels).
static ocfd_status chem_half(ocfd_react* R, cudaStream_t st, int& launches, bool last, bool& renormed) {
    renormed = false;
    ocfd_level* L = R->L;
    const double dt2 = 0.5 * R->desc.dt / R->desc.chem_substeps;
    const int sms = R->ctx->num_sms;
    if (R->mlp) {
        // network substep over the level's cells, then the FP64 substep for the
        // cells the guard rejected
        for (int s = 0; s < R->desc.chem_substeps; ++s) {
            cudaMemsetAsync(R->fb_count, 0, sizeof(unsigned), st);
            ocfd_status r = launch_chem_surrogate(R->mlp, R->off, R->stride, R->nactive, L->buf[0], dt2, R->ctx->parm,
                                                  R->guard, R->fb_off, R->fb_stride, R->fb_count, R->fb_total,
                                                  R->ctx->d_error, sms, st);
            if (r == OCFD_OK)
                r = launch_chem_advance_list(R->fb_off, R->fb_stride, L->ncells, L->buf[0], dt2, R->ctx->parm, st,
                                             R->fb_count, nullptr);
            if (r != OCFD_OK) return r;
            launches += 2;
        }
        return OCFD_OK;
    }
    if (R->desc.binned_chem) {
        cudaMemsetAsync(R->count, 0, sizeof(unsigned) * NBIN, st);
        if (R->nactive == 0) return OCFD_OK;
        k_react_keys<<<grid_for(R->nactive, 256, sms), 256, 0, st>>>(R->d_afabs, R->d_astart, R->nabox, R->nactive,
                                                                    L->buf[0], R->a0w, R->key, R->count);
        k_react_scan<<<1, 1, 0, st>>>(R->count);
        k_react_scatter<<<grid_for(R->nactive, 256, sms), 256, 0, st>>>(R->d_afabs, R->d_astart, R->nabox, R->nactive,
                                                                       R->key, R->count, R->off, R->stride);
        launches += 3;
        for (int s = 0; s < R->desc.chem_substeps; ++s) {
            const bool rn = last && s == R->desc.chem_substeps - 1;
            ocfd_status r = launch_chem_advance_list(R->off, R->stride, R->nactive, L->buf[0], dt2, R->ctx->parm, st,
                                                     nullptr, nullptr, rn);
            if (r != OCFD_OK) return r;
            ++launches;
        }
        renormed = last && R->desc.chem_substeps > 0;
        return OCFD_OK;
    }
    renormed = last && R->desc.chem_substeps > 0;
    for (int s = 0; s < R->desc.chem_substeps; ++s)
        for (size_t b = 0; b < L->boxes.size(); ++b) {
            if (!R->cls.empty() && R->cls[b] == OCFD_BOX_COVERED) continue;
            ocfd_array4 S = fab_view(L, L->buf[0], (int)b, 0, 5), sp = fab_view(L, L->buf[0], (int)b, 5, NSP);
            CellBox cb{};
            for (int d = 0; d < 3; ++d) {
                cb.lo[d] = L->boxes[b].lo[d];
                cb.n[d] = L->boxes[b].hi[d] - L->boxes[b].lo[d] + 1;
            }
            ocfd_status r = launch_chem_advance(view_of<double>(&S), view_of<double>(&sp), cb, dt2, R->ctx->parm, st,
                                                last && s == R->desc.chem_substeps - 1);
            if (r != OCFD_OK) return r;
            ++launches;
        }
    return OCFD_OK;
}

// The RHS argument blocks of every box for each stage input buffer: the regular
// chain, or for a cut box the cut-cell chain on the level's geometry
static void build_args(ocfd_react* R) {
    ocfd_level* L = R->L;
    const double dxinv[3] = {1.0 / L->desc.dx[0], 1.0 / L->desc.dx[1], 1.0 / L->desc.dx[2]};
    for (int in = 0; in < 3; ++in) {
        R->args[in].clear();
        for (size_t b = 0; b < L->boxes.size(); ++b) {
            ocfd_array4 S = fab_view(L, L->buf[in], (int)b, 0, 5), sp = fab_view(L, L->buf[in], (int)b, 5, NSP);
            ocfd_array4 d = fab_view(L, R->rhs, (int)b, 0, 5), ds = fab_view(L, R->rhs, (int)b, 5, NSP);
            ChemBoxArgs A{};
            chem_rhs_args(A, view_of<const double>(&S), view_of<const double>(&sp), view_of<double>(&d),
                          view_of<double>(&ds), L->boxes[b], dxinv, (R->desc.flags & OCFD_VISC) != 0, R->scr);
            A.f32 = (R->desc.flags & OCFD_FLUX_FP32) ? 1 : 0;
            if (!R->cls.empty() && R->cls[b] == OCFD_BOX_CUT) {
                View<const uint32_t> fl;
                View<const double> vf, ap[3];
                if (eb_box_views(L, (int)b, fl, vf, ap)) chem_args_as_cut(A, fl, vf, ap);
            }
            R->args[in].push_back(A);
        }
    }
}

// The boxes the chemistry visits (all but the covered ones), their cells, and
// the identity cell list over them (re-ordered by the binned form every half step)
static ocfd_status build_active(ocfd_react* R) {
    ocfd_level* L = R->L;
    cudaFree(R->d_afabs);
    cudaFree(R->d_astart);
    R->d_afabs = nullptr;
    R->d_astart = nullptr;
    std::vector<FabGeom> af;
    std::vector<long long> as;
    long long n = 0;
    for (size_t b = 0; b < L->boxes.size(); ++b) {
        if (!R->cls.empty() && R->cls[b] == OCFD_BOX_COVERED) continue;
        af.push_back(L->fabs[b]);
        as.push_back(n);
        n += region_cells(L->fabs[b].lo, L->fabs[b].hi);
    }
    ocfd_status s = upload(&R->d_afabs, af);
    if (s == OCFD_OK) s = upload(&R->d_astart, as);
    if (s != OCFD_OK) return s;
    R->nabox = (int)af.size();
    R->nactive = n;
    if (n > 0)
        k_react_identity<<<grid_for(n, 256, R->ctx->num_sms), 256>>>(R->d_afabs, R->d_astart, R->nabox, n, R->off,
                                                                    R->stride);
    return check_launch("reacting level cell list");
}

static ocfd_status record_react_step(ocfd_react* R, unsigned flags, cudaStream_t st) {
    (void)flags;
    ocfd_level* L = R->L;
    int launches = 0;
    k_react_begin<<<1, 1, 0, st>>>(L->d_step, R->desc.dt);
    ++launches;
    bool renormed = false;
    ocfd_status s = chem_half(R, st, launches, false, renormed);
    if (s != OCFD_OK) return s;
    // flow: stage k reads buffer in[k], writes out[k] = a U^n + b (in + dt L(in))
    const bool rk3 = R->desc.rk_order == 3;
    const int nst = rk3 ? 3 : 2;
    const int in3[3] = {0, 1, 2}, out3[3] = {1, 2, 0};
    const int in2[2] = {0, 1}, out2[2] = {1, 0};
    const double a3[3] = {0.0, 0.75, 1.0 / 3.0}, b3[3] = {1.0, 0.25, 2.0 / 3.0};
    const double a2[2] = {0.0, 0.5}, b2[2] = {1.0, 0.5};
    const double tf3[3] = {0.0, 1.0, 0.5}, tf2[2] = {0.0, 1.0};
    const int sms = R->ctx->num_sms;
    for (int k = 0; k < nst && s == OCFD_OK; ++k) {
        const int in = rk3 ? in3[k] : in2[k], out = rk3 ? out3[k] : out2[k];
        s = fill_ghosts(L, L->buf[in], rk3 ? tf3[k] : tf2[k], st, true);
        launches += (L->ex_total > 0) + (L->bc_total[0] > 0) + (L->bc_total[1] > 0) + (L->bc_total[2] > 0);
        for (size_t b = 0; b < L->boxes.size() && s == OCFD_OK; ++b) {
            const ChemBoxArgs& A = R->args[in][b];
            if (!R->cls.empty() && R->cls[b] == OCFD_BOX_COVERED) continue;  // dSdt = 0 (Advance.cpp:213-214)
            s = A.eb ? launch_chem_eb_rhs(A, R->ctx->parm, sms, st) : launch_chem_rhs(A, R->ctx->parm, sms, st);
            launches += A.visc ? 6 : 5;
        }
        if (s != OCFD_OK) break;
        k_react_combine<<<grid_for(L->ncells, 256, sms), 256, 0, st>>>(
            L->d_fabs, L->d_cell_start, (int)L->boxes.size(), L->ncells, L->buf[out], L->buf[0], L->buf[in], R->rhs,
            rk3 ? a3[k] : a2[k], rk3 ? b3[k] : b2[k], L->d_step);
        ++launches;
        s = check_launch("reacting flow stage");
    }
    if (s != OCFD_OK) return s;
    s = chem_half(R, st, launches, true, renormed);
    if (s != OCFD_OK) return s;
    // species renormalisation of the cells the chemistry did not finish (every
    // cell in the surrogate form; the covered boxes of a level with a body)
    for (size_t b = 0; b < L->boxes.size(); ++b) {
        if (renormed && (R->cls.empty() || R->cls[b] != OCFD_BOX_COVERED)) continue;
        ocfd_array4 S = fab_view(L, L->buf[0], (int)b, 0, 5), sp = fab_view(L, L->buf[0], (int)b, 5, NSP);
        CellBox cb{};
        for (int d = 0; d < 3; ++d) {
            cb.lo[d] = L->boxes[b].lo[d];
            cb.n[d] = L->boxes[b].hi[d] - L->boxes[b].lo[d] + 1;
        }
        s = launch_spec_renorm(view_of<const double>(&S), view_of<double>(&sp), cb, sms, st);
        if (s != OCFD_OK) return s;
        ++launches;
    }
    k_react_end<<<1, 1, 0, st>>>(L->d_step);
    ++launches;
    R->launches = launches;
    return check_launch("reacting step");
}

}  // namespace ocfd

using namespace ocfd;

extern "C" {

ocfd_status ocfd_react_create(ocfd_context* ctx, const ocfd_react_desc* desc, ocfd_react** out) {
    if (!ctx || !desc || !out) return fail(OCFD_BAD_ARG, "ocfd_react_create: bad arguments");
    *out = nullptr;
    if (desc->rk_order != 2 && desc->rk_order != 3) return fail(OCFD_BAD_ARG, "ocfd_react_create: rk_order is 2 or 3");
    if (desc->chem_substeps < 0 || !(desc->dt > 0)) return fail(OCFD_BAD_ARG, "ocfd_react_create: substeps / dt");
    ocfd_react* R = new ocfd_react();
    R->ctx = ctx;
    R->desc = *desc;
    R->desc.level.boxes = nullptr;
    ocfd_status s = level_alloc(ctx, &desc->level, 3, &R->L, nullptr, NCOMP_REACT);
    if (s != OCFD_OK) {
        delete R;
        return s;
    }
    ocfd_level* L = R->L;
    size_t scr = 0;
    for (const ocfd_box& b : L->boxes) scr = std::max(scr, chem_rhs_scratch_doubles(b));
    if (cudaMalloc(&R->rhs, sizeof(double) * L->elems) != cudaSuccess ||
        cudaMalloc(&R->scr, sizeof(double) * scr) != cudaSuccess ||
        cudaMalloc(&R->key, std::max<long long>(1, L->ncells)) != cudaSuccess ||
        cudaMalloc(&R->count, sizeof(unsigned) * NBIN) != cudaSuccess ||
        cudaMalloc(&R->off, sizeof(long long) * std::max<long long>(1, L->ncells)) != cudaSuccess ||
        cudaMalloc(&R->stride, sizeof(long long) * std::max<long long>(1, L->ncells)) != cudaSuccess ||
        cudaMalloc(&R->a0w, sizeof(double) * NSP) != cudaSuccess) {
        cudaGetLastError();
        ocfd_react_destroy(R);
        return fail(OCFD_OUT_OF_MEMORY, "ocfd_react_create: buffers");
    }
    cudaMemset(R->rhs, 0, sizeof(double) * L->elems);
    if (cudaMalloc(&R->fb_off, sizeof(long long) * std::max<long long>(1, L->ncells)) != cudaSuccess ||
        cudaMalloc(&R->fb_stride, sizeof(long long) * std::max<long long>(1, L->ncells)) != cudaSuccess ||
        cudaMalloc(&R->fb_count, sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc(&R->fb_total, sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        ocfd_react_destroy(R);
        return fail(OCFD_OUT_OF_MEMORY, "ocfd_react_create: fallback list");
    }
    cudaMemset(R->fb_total, 0, sizeof(unsigned long long));
    s = build_active(R);
    if (s != OCFD_OK) {
        ocfd_react_destroy(R);
        return s;
    }
    // (a0 - 1) Ru / W_i of the Newton start (LiDryer.H:833-888)
    {
        MechTables t;
        mech_builtin(&t);
        ocfd_parm hp = ctx->host_parm;
        double a0w[NSP];
        for (int n = 0; n < NSP; ++n) a0w[n] = t.A0[n] * hp.Ru / t.mw[n];
        cudaMemcpy(R->a0w, a0w, sizeof(a0w), cudaMemcpyHostToDevice);
    }
    build_args(R);
    if (cudaDeviceSynchronize() != cudaSuccess) {
        ocfd_react_destroy(R);
        return check_launch("ocfd_react_create");
    }
    *out = R;
    return OCFD_OK;
}

ocfd_status ocfd_react_destroy(ocfd_react* R) {
    if (!R) return OCFD_OK;
    if (R->graph) cudaGraphExecDestroy(R->graph);
    cudaFree(R->rhs);
    cudaFree(R->scr);
    cudaFree(R->key);
    cudaFree(R->count);
    cudaFree(R->off);
    cudaFree(R->stride);
    cudaFree(R->a0w);
    cudaFree(R->fb_off);
    cudaFree(R->fb_stride);
    cudaFree(R->fb_count);
    cudaFree(R->fb_total);
    cudaFree(R->d_afabs);
    cudaFree(R->d_astart);
    if (R->L) ocfd_level_destroy(R->L);
    delete R;
    return OCFD_OK;
}

ocfd_level* ocfd_react_level(ocfd_react* R) { return R ? R->L : nullptr; }

ocfd_status ocfd_react_advance(ocfd_react* R, int nsteps, void* stream) {
    if (!R || nsteps < 0) return fail(OCFD_BAD_ARG, "ocfd_react_advance");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (nsteps == 0) return OCFD_OK;
    if (!R->graph) {
        cudaStream_t cap;
        if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return check_launch("capture stream");
        cudaGraph_t g;
        if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaStreamDestroy(cap);
            return check_launch("begin capture");
        }
        ocfd_status s = record_react_step(R, 0, cap);
        cudaError_t e = cudaStreamEndCapture(cap, &g);
        cudaStreamDestroy(cap);
        if (s != OCFD_OK) return s;
        if (e != cudaSuccess) return fail(OCFD_LAUNCH_FAIL, std::string("end capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&R->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(OCFD_LAUNCH_FAIL, std::string("graph instantiate: ") + cudaGetErrorString(e));
    }
    for (int i = 0; i < nsteps; ++i)
        if (cudaGraphLaunch(R->graph, st) != cudaSuccess) return check_launch("reacting graph launch");
    return OCFD_OK;
}

int ocfd_react_launches_per_step(const ocfd_react* R) { return R ? R->launches : 0; }

ocfd_status ocfd_react_set_surrogate(ocfd_react* R, ocfd_mlp* mlp, const ocfd_surrogate_guard* guard) {
    if (!R || (mlp && !guard)) return fail(OCFD_BAD_ARG, "ocfd_react_set_surrogate");
    R->mlp = mlp;
    if (guard) R->guard = *guard;
    if (R->graph) {
        cudaGraphExecDestroy(R->graph);
        R->graph = nullptr;
    }
    return OCFD_OK;
}

ocfd_status ocfd_react_fallbacks(ocfd_react* R, int64_t* fallbacks, void* stream) {
    if (!R || !fallbacks) return fail(OCFD_BAD_ARG, "ocfd_react_fallbacks");
    unsigned long long h = 0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemcpyAsync(&h, R->fb_total, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return check_launch("ocfd_react_fallbacks");
    *fallbacks = (int64_t)h;
    return OCFD_OK;
}

ocfd_status ocfd_react_set_eb(ocfd_react* R, const ocfd_eb_desc* eb) {
    if (!R || !eb) return fail(OCFD_BAD_ARG, "ocfd_react_set_eb: null argument");
    if (cudaDeviceSynchronize() != cudaSuccess) return check_launch("ocfd_react_set_eb");
    ocfd_level* L = R->L;
    ocfd_status s = eb_setup(L, *eb);
    if (s != OCFD_OK) return s;
    R->cls.clear();
    if (eb->kind != OCFD_EB_NONE)
        for (size_t b = 0; b < L->boxes.size(); ++b) R->cls.push_back(eb_box_class(L, (int)b));
    // covered boxes keep a zero right-hand side
    if (cudaMemset(R->rhs, 0, sizeof(double) * L->elems) != cudaSuccess) return check_launch("ocfd_react_set_eb");
    build_args(R);
    s = build_active(R);
    if (R->graph) {
        cudaGraphExecDestroy(R->graph);
        R->graph = nullptr;
    }
    if (s == OCFD_OK && cudaDeviceSynchronize() != cudaSuccess) s = check_launch("ocfd_react_set_eb");
    return s;
}

ocfd_status ocfd_react_box_classes(const ocfd_react* R, int32_t* cls) {
    if (!R || !cls) return fail(OCFD_BAD_ARG, "ocfd_react_box_classes");
    for (size_t b = 0; b < R->L->boxes.size(); ++b) cls[b] = R->cls.empty() ? OCFD_BOX_REGULAR : R->cls[b];
    return OCFD_OK;
}

ocfd_status ocfd_react_profile_chem(ocfd_react* R, int reps, double* ms, void* stream) {
    if (!R || reps <= 0 || !ms) return fail(OCFD_BAD_ARG, "ocfd_react_profile_chem");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    ocfd_react_desc d = R->desc;
    R->desc.chem_substeps = 1;
    int launches = 0;
    bool rn = false;
    ocfd_status s = chem_half(R, st, launches, false, rn);  // warm-up
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    for (int r = 0; r < reps && s == OCFD_OK; ++r) s = chem_half(R, st, launches, false, rn);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    R->desc = d;
    *ms = t / reps;
    return s;
}

}  // extern "C"
