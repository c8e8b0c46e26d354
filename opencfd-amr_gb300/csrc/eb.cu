// Cut-cell box right-hand side (ideal gas), replacing the kernel chain of
// EBR::eb_compute_dSdt_box (Source/EB/AdvanceBox.cpp:78-214):
//   k_eb_prims      primitives over grow(bx, 2)               (c2prim)
//   k_eb_faces<D>   per face: MUSCL-minmod left/right states of the 7
//                   primitives, Van Leer flux, EB viscous flux (eb_recon_*,
//                   eb_flux, eb_compute_visc_*), written to the face array
//   k_eb_div        per cell: cut-cell divergence with the wall flux, negated,
//                   optional local rescale (eb_compute_div(_visc), flux_redist)
// The reference stages ql/qr over the whole nodal box in HBM; here they live
// in registers of the face thread.
#include <cuda_runtime.h>

#include <string>

#include "eb_physics.cuh"
#include "ocfd_internal.h"

namespace ocfd {

struct EbBoxArgs {
    View<const double> S;
    View<double> dsdt;
    View<double> flux[3];
    View<const uint32_t> flag;
    View<const double> vfrac;
    View<const double> ap[3];
    View<double> q;  // scratch primitives over grow(bx, 2)
    int lo[3], hi[3];
    double dxinv[3];
    int visc, redist;
};

__global__ void k_eb_prims(EbBoxArgs B, DevParm P) {
    const int gx = B.hi[0] - B.lo[0] + 5, gy = B.hi[1] - B.lo[1] + 5, gz = B.hi[2] - B.lo[2] + 5;
    const long long n = (long long)gx * gy * gz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        const int i = B.lo[0] - 2 + (int)(c % gx), j = B.lo[1] - 2 + (int)((c / gx) % gy),
                  k = B.lo[2] - 2 + (int)(c / ((long long)gx * gy));
        double q[7];
        c2prim_ideal_fast(P, B.S(i, j, k, 0), B.S(i, j, k, 1), B.S(i, j, k, 2), B.S(i, j, k, 3),
                     B.S(i, j, k, 4), q);
#pragma unroll
        for (int m = 0; m < 7; ++m) B.q(i, j, k, m) = q[m];
    }
}

template <int D>
__global__ void k_eb_faces(EbBoxArgs B, DevParm P) {
    const int fx = B.hi[0] - B.lo[0] + 1 + (D == 0), fy = B.hi[1] - B.lo[1] + 1 + (D == 1),
              fz = B.hi[2] - B.lo[2] + 1 + (D == 2);
    const long long n = (long long)fx * fy * fz;
    const int di = D == 0, dj = D == 1, dk = D == 2;
    const View<const double> q{B.q.p, B.q.js, B.q.ks, B.q.ns, B.q.b0, B.q.b1, B.q.b2};
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        const int i = B.lo[0] + (int)(c % fx), j = B.lo[1] + (int)((c / fx) % fy),
                  k = B.lo[2] + (int)(c / ((long long)fx * fy));
        const uint32_t f = B.flag(i, j, k);
        double ql[7], qr[7];
#pragma unroll
        for (int m = 0; m < 7; ++m) {
            if (m == QT) {  // the Van Leer flux does not read the temperature
                ql[m] = qr[m] = 0.0;
                continue;
            }
            eb_recon(f, D, q(i - 2 * di, j - 2 * dj, k - 2 * dk, m), q(i - di, j - dj, k - dk, m),
                     q(i, j, k, m), q(i + di, j + dj, k + dk, m), ql[m], qr[m]);
        }
        double flx[5];
        vanleer_g<double>(P.smallp, P.gamma, P.vl_rg, P.vl_rg21, P.vl_ggm1, ql, qr, D, flx);
        if (B.visc) eb_visc_face(P, q, B.flag, D, i, j, k, B.dxinv, flx, 1, false, 0, 0, 0);
#pragma unroll
        for (int m = 0; m < 5; ++m) B.flux[D](i, j, k, m) = flx[m];
    }
}

// one cut-cell divergence (Source/EB/EBkernels.H:216-338), negated
__global__ void k_eb_div(EbBoxArgs B, DevParm P) {
    const int nx = B.hi[0] - B.lo[0] + 1, ny = B.hi[1] - B.lo[1] + 1, nz = B.hi[2] - B.lo[2] + 1;
    const long long n = (long long)nx * ny * nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        const int i = B.lo[0] + (int)(c % nx), j = B.lo[1] + (int)((c / nx) % ny),
                  k = B.lo[2] + (int)(c / ((long long)nx * ny));
        const uint32_t f = B.flag(i, j, k);
        const double vf = B.vfrac(i, j, k);
        const double tmp = B.dxinv[0] / vf;
        double out[5];
        if (eb_covered(f)) {
#pragma unroll
            for (int m = 0; m < 5; ++m) out[m] = 0.0;
        } else if (eb_regular(f)) {
#pragma unroll
            for (int m = 0; m < 5; ++m)
                out[m] = B.dxinv[0] * (B.flux[0](i + 1, j, k, m) - B.flux[0](i, j, k, m)) +
                         B.dxinv[1] * (B.flux[1](i, j + 1, k, m) - B.flux[1](i, j, k, m)) +
                         B.dxinv[2] * (B.flux[2](i, j, k + 1, m) - B.flux[2](i, j, k, m));
        } else {
            const double axm = B.ap[0](i, j, k), axp = B.ap[0](i + 1, j, k);
            const double aym = B.ap[1](i, j, k), ayp = B.ap[1](i, j + 1, k);
            const double azm = B.ap[2](i, j, k), azp = B.ap[2](i, j, k + 1);
#pragma unroll
            for (int m = 0; m < 5; ++m)
                out[m] = tmp * (axp * B.flux[0](i + 1, j, k, m) - axm * B.flux[0](i, j, k, m) +
                                ayp * B.flux[1](i, j + 1, k, m) - aym * B.flux[1](i, j, k, m) +
                                azp * B.flux[2](i, j, k + 1, m) - azm * B.flux[2](i, j, k, m));
            double fw[5];
            const double pr = B.q(i, j, k, QPRES);
            if (!B.visc) {
                // slip-wall pressure flux, EBkernels.H:305-311
                fw[0] = 0.0;
                fw[1] = (axm - axp) * pr;
                fw[2] = (aym - ayp) * pr;
                fw[3] = (azm - azp) * pr;
                fw[4] = 0.0;
            } else {
                // eb_wallflux, EBkernels.H:173-214
                const double d = B.q(i, j, k, QRHO), u = B.q(i, j, k, QU), v = B.q(i, j, k, QV),
                             w = B.q(i, j, k, QW), cs = B.q(i, j, k, QC);
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
        const bool rescale = B.redist && vf < 0.5 && vf > 0.0;
#pragma unroll
        for (int m = 0; m < 5; ++m) {
            const double divc = out[m] * -1.0;
            B.dsdt(i, j, k, m) = rescale ? vf * divc : divc;
        }
    }
}

static int blocks_for(long long n, int threads, int sms) {
    long long b = (n + threads - 1) / threads;
    long long cap = (long long)sms * 32;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace ocfd

using namespace ocfd;

namespace ocfd {

// Argument checks and scratch size of one cut-cell box (shared by both entry
// points, so that they accept and reject exactly the same boxes).
struct EbBoxPlan {
    int n[3];
    long long gcells, fcells[3];
    long long need;  // scratch doubles: primitives over grow(bx, 2), + face fluxes without `flux`
};

static ocfd_status eb_box_check(const char* who, ocfd_context* ctx, const ocfd_array4* S,
                                const ocfd_array4* dSdt, const ocfd_array4* flux, const ocfd_flag4* flag,
                                const ocfd_array4* vfrac, const ocfd_array4* const ap[3], ocfd_box bx,
                                const double dxinv[3], unsigned flags, EbBoxPlan* plan) {
    const std::string w(who);
    if (!ctx || !dxinv) return fail(OCFD_BAD_ARG, w + ": null argument");
    for (int d = 0; d < 3; ++d)
        if (bx.hi[d] < bx.lo[d]) return fail(OCFD_BAD_ARG, w + ": empty box");
    if (!covers(S, bx, 2, 5)) return fail(OCFD_BAD_ARG, w + ": S must cover grow(bx,2)");
    if (!covers(dSdt, bx, 0, 5)) return fail(OCFD_BAD_ARG, w + ": dSdt must cover bx");
    if (!covers_flag(flag, bx, 1)) return fail(OCFD_BAD_ARG, w + ": flag must cover grow(bx,1)");
    if (!covers(vfrac, bx, 0, 1)) return fail(OCFD_BAD_ARG, w + ": vfrac must cover bx");
    for (int d = 0; d < 3; ++d)
        if (!covers(ap[d], bx, 0, 1, d))
            return fail(OCFD_BAD_ARG, w + ": area fractions must cover surroundingNodes(bx,d)");
    if (flux)
        for (int d = 0; d < 3; ++d)
            if (!covers(&flux[d], bx, 0, 5, d)) return fail(OCFD_BAD_ARG, w + ": flux[d]");
    if (flags & ~(unsigned)(OCFD_VISC | OCFD_REDISTRIBUTE)) return fail(OCFD_BAD_ARG, w + ": unsupported flags");
    for (int d = 0; d < 3; ++d) plan->n[d] = bx.hi[d] - bx.lo[d] + 1;
    const int* n = plan->n;
    plan->gcells = (long long)(n[0] + 4) * (n[1] + 4) * (n[2] + 4);
    for (int d = 0; d < 3; ++d)
        plan->fcells[d] = (long long)(n[0] + (d == 0)) * (n[1] + (d == 1)) * (n[2] + (d == 2));
    plan->need = 7 * plan->gcells;
    if (!flux) plan->need += 5 * (plan->fcells[0] + plan->fcells[1] + plan->fcells[2]);
    return OCFD_OK;
}

// The kernel chain of one cut-cell box (primitives, three face passes,
// divergence) with its scratch at `scr` (plan.need doubles).
static ocfd_status eb_box_launch(const char* who, ocfd_context* ctx, const ocfd_array4* S,
                                 const ocfd_array4* dSdt, const ocfd_array4* flux, const ocfd_flag4* flag,
                                 const ocfd_array4* vfrac, const ocfd_array4* const ap[3], ocfd_box bx,
                                 const double dxinv[3], unsigned flags, const EbBoxPlan& plan, double* scr,
                                 void* stream) {
    const int* n = plan.n;
    EbBoxArgs B{};
    B.S = view_of<const double>(S);
    B.dsdt = view_of<double>(dSdt);
    B.flag = view_of_flag(flag);
    B.vfrac = view_of<const double>(vfrac);
    for (int d = 0; d < 3; ++d) {
        B.ap[d] = view_of<const double>(ap[d]);
        B.lo[d] = bx.lo[d];
        B.hi[d] = bx.hi[d];
        B.dxinv[d] = dxinv[d];
    }
    B.q = View<double>{scr, n[0] + 4, (long long)(n[0] + 4) * (n[1] + 4), plan.gcells,
                       bx.lo[0] - 2, bx.lo[1] - 2, bx.lo[2] - 2};
    double* fp = scr + 7 * plan.gcells;
    for (int d = 0; d < 3; ++d) {
        if (flux) {
            B.flux[d] = view_of<double>(&flux[d]);
        } else {
            const int sx = n[0] + (d == 0), sy = n[1] + (d == 1);
            B.flux[d] = View<double>{fp, sx, (long long)sx * sy, plan.fcells[d], bx.lo[0], bx.lo[1], bx.lo[2]};
            fp += 5 * plan.fcells[d];
        }
    }
    B.visc = (flags & OCFD_VISC) != 0;
    B.redist = (flags & OCFD_REDISTRIBUTE) != 0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int T = 256, sms = ctx->num_sms;
    k_eb_prims<<<blocks_for(plan.gcells, T, sms), T, 0, st>>>(B, ctx->parm);
    k_eb_faces<0><<<blocks_for(plan.fcells[0], T, sms), T, 0, st>>>(B, ctx->parm);
    k_eb_faces<1><<<blocks_for(plan.fcells[1], T, sms), T, 0, st>>>(B, ctx->parm);
    k_eb_faces<2><<<blocks_for(plan.fcells[2], T, sms), T, 0, st>>>(B, ctx->parm);
    k_eb_div<<<blocks_for((long long)n[0] * n[1] * n[2], T, sms), T, 0, st>>>(B, ctx->parm);
    return check_launch(who);
}

}  // namespace ocfd

extern "C" ocfd_status ocfd_rhs_eb_box_f64(ocfd_context* ctx, const ocfd_array4* S,
                                           const ocfd_array4* dSdt, const ocfd_array4* flux,
                                           const ocfd_flag4* flag, const ocfd_array4* vfrac,
                                           const ocfd_array4* apx, const ocfd_array4* apy,
                                           const ocfd_array4* apz, const ocfd_array4* const* fc,
                                           const ocfd_array4* bcent, ocfd_box bx,
                                           const double dxinv[3], unsigned flags, void* stream) {
    (void)fc;
    (void)bcent;
    const char* who = "ocfd_rhs_eb_box_f64";
    const ocfd_array4* ap[3] = {apx, apy, apz};
    EbBoxPlan plan{};
    ocfd_status s = eb_box_check(who, ctx, S, dSdt, flux, flag, vfrac, ap, bx, dxinv, flags, &plan);
    if (s != OCFD_OK) return s;
    double* scr = static_cast<double*>(scratch(ctx, sizeof(double) * (size_t)plan.need));
    if (!scr) return fail(OCFD_OUT_OF_MEMORY, std::string(who) + ": scratch");
    return eb_box_launch(who, ctx, S, dSdt, flux, flag, vfrac, ap, bx, dxinv, flags, plan, scr, stream);
}

// ---------------------------------------------------------------------------
// Allocation-free variant of ocfd_rhs_eb_box_f64.
//
// Some callers cannot let a library allocate device memory: applications that
// hand all device memory to their own pool (an AMReX arena sized at start-up,
// a memory-capped service) and must not see allocations appear behind their
// back, and code paths where a cudaMalloc / cudaFree - which can synchronise
// the whole device - would stall other streams at the wrong moment.  This
// variant runs the same kernel chain as ocfd_rhs_eb_box_f64 (primitives, three
// face passes, divergence) but takes its scratch (cell primitives, and the face
// fluxes when the caller passes no flux arrays) from a fixed array compiled
// into the library, so it allocates nothing at any call.
//
// The array is kEbStaticScratchDoubles doubles (16 MiB) and is held by every
// GPU that loads the library until the process exits.  Its device address is
// looked up when a context is created (eb_static_scratch_resolve, called by
// ocfd_context_create with the context's device current); that lookup loads
// this file's device code, so the array is resident before the first call and
// no call can trigger a lazy module load.  All calls share it and it keeps
// whatever the last call left there: calls that overlap on the GPU (different
// streams, or different host threads) race on it and must be serialised by
// the caller.  Nothing in it has to start at zero - every value a kernel reads
// was written earlier in the same call.
// ---------------------------------------------------------------------------
namespace ocfd {

constexpr long long kEbStaticScratchDoubles = 2LL * 1024 * 1024;

static __device__ __align__(256) double g_eb_static_scratch[kEbStaticScratchDoubles];

// In host code g_eb_static_scratch names a host-side stand-in, not the device
// array: a kernel must be given the address cudaGetSymbolAddress returns.
// With lazy module loading the lookup also loads this file's device code, and
// the attribute queries load the five kernels of the chain, so that no later
// call has code or data of this file to bring onto the device.
ocfd_status eb_static_scratch_resolve(ocfd_context* ctx) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_eb_static_scratch);
    cudaFuncAttributes fa;
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_eb_prims);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_eb_faces<0>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_eb_faces<1>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_eb_faces<2>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_eb_div);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return fail(OCFD_LAUNCH_FAIL, std::string("static scratch: device code of the cut-cell box not loadable: ") +
                                          cudaGetErrorString(e));
    }
    ctx->eb_static_scratch = static_cast<double*>(p);
    return OCFD_OK;
}

}  // namespace ocfd

extern "C" ocfd_status ocfd_rhs_eb_box_f64_static_scratch(
    ocfd_context* ctx, const ocfd_array4* S, const ocfd_array4* dSdt, const ocfd_array4* flux,
    const ocfd_flag4* flag, const ocfd_array4* vfrac, const ocfd_array4* apx, const ocfd_array4* apy,
    const ocfd_array4* apz, const ocfd_array4* const* fc, const ocfd_array4* bcent, ocfd_box bx,
    const double dxinv[3], unsigned flags, void* stream) {
    (void)fc;
    (void)bcent;
    const char* who = "ocfd_rhs_eb_box_f64_static_scratch";
    const ocfd_array4* ap[3] = {apx, apy, apz};
    EbBoxPlan plan{};
    ocfd_status s = eb_box_check(who, ctx, S, dSdt, flux, flag, vfrac, ap, bx, dxinv, flags, &plan);
    if (s != OCFD_OK) return s;
    if (plan.need > kEbStaticScratchDoubles)
        return fail(OCFD_BAD_ARG, std::string(who) + ": box needs " + std::to_string(plan.need) +
                                      " scratch doubles, the static scratch holds " +
                                      std::to_string(kEbStaticScratchDoubles) +
                                      " (pass flux arrays or split the box)");
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return check_launch(who);
    if (dev != ctx->device)
        return fail(OCFD_BAD_ARG, std::string(who) + ": the context's device must be the current device");
    if (!ctx->eb_static_scratch) return fail(OCFD_LAUNCH_FAIL, std::string(who) + ": static scratch not resolved");
    return eb_box_launch(who, ctx, S, dSdt, flux, flag, vfrac, ap, bx, dxinv, flags, plan, ctx->eb_static_scratch,
                         stream);
}
