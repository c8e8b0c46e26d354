// Li-Dryer chemistry on the GPU: mechanism tables in constant memory and the
// kernels that read them (real-gas primitives, transport, multispecies RHS,
// implicit chemistry substep).
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "chem_physics.cuh"
#include "mechanism.h"
#include "ocfd_internal.h"

namespace ocfd {

void mech_builtin(MechTables* t);

ocfd_status mech_upload(const ocfd_parm& p) {
    MechTables t;
    mech_builtin(&t);
    auto fetch = [](double* dst, const double* src, size_t n) -> bool {
        if (!src) return true;
        return cudaMemcpy(dst, src, n * sizeof(double), cudaMemcpyDefault) == cudaSuccess;
    };
    const double* lo[NSP] = {p.H2_lo, p.O2_lo, p.H2O_lo, p.H_lo, p.O_lo, p.OH_lo, p.HO2_lo, p.H2O2_lo, p.N2_lo};
    const double* hi[NSP] = {p.H2_hi, p.O2_hi, p.H2O_hi, p.H_hi, p.O_hi, p.OH_hi, p.HO2_hi, p.H2O2_hi, p.N2_hi};
    bool ok = fetch(t.mw, p.mw, NSP);
    for (int n = 0; n < NSP; ++n) ok = ok && fetch(t.lo[n], lo[n], 7) && fetch(t.hi[n], hi[n], 7);
    ok = ok && fetch(t.HP, p.HP, NSP) && fetch(t.A0, p.A0, NSP) && fetch(t.visc, p.visccoeff, NSP * 5) &&
         fetch(t.cond, p.conductcoeff, NSP * 5) && fetch(t.diff, p.diffcoeff, 45 * 5);
    if (!ok) {
        cudaGetLastError();
        return fail(OCFD_BAD_ARG, "mechanism tables: cannot read the Parm table pointers");
    }
    if (cudaMemcpyToSymbol(c_mech, &t, sizeof(t)) != cudaSuccess) {
        cudaError_t e = cudaGetLastError();
        return fail(OCFD_LAUNCH_FAIL, std::string("mechanism upload: ") + cudaGetErrorString(e));
    }
    return OCFD_OK;
}

// Per-thread 9x10 matrix in shared memory, element-major so that the threads
// of a warp touch consecutive words.
struct SmemMat {
    double* base;
    int stride;
    __device__ __forceinline__ double& operator()(int r, int c) const { return base[(r * 10 + c) * stride]; }
};

struct CellBox {
    int lo[3], n[3];
    __device__ __forceinline__ long long count() const { return (long long)n[0] * n[1] * n[2]; }
    __device__ __forceinline__ void cell(long long c, int& i, int& j, int& k) const {
        i = lo[0] + (int)(c % n[0]);
        j = lo[1] + (int)((c / n[0]) % n[1]);
        k = lo[2] + (int)(c / ((long long)n[0] * n[1]));
    }
};

constexpr int kChemThreads = 128;

// One semi-implicit chemistry substep per cell, in place: the lambda of
// EBR::chemical_advance, Source/CHEM/ChemAdvance.cpp:27-82.
__global__ void __launch_bounds__(kChemThreads) k_chem_advance(View<double> S, View<double> sp, CellBox B,
                                                               double dt, DevParm P) {
    extern __shared__ double smem[];
    const SmemMat U{smem + threadIdx.x, (int)blockDim.x};
    const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (c >= B.count()) return;
    int i, j, k;
    B.cell(c, i, j, k);
    const double rho = dmax(S(i, j, k, 0), P.smallr);
    const double rhoinv = 1.0 / rho;
    const double ux = S(i, j, k, 1) * rhoinv, uy = S(i, j, k, 2) * rhoinv, uz = S(i, j, k, 3) * rhoinv;
    const double kineng = 0.5 * (ux * ux + uy * uy + uz * uz);
    const double ei = S(i, j, k, 4) - rho * kineng;
    double r0[NSP], cc[NSP], wdot[NSP], drho[NSP];
#pragma unroll
    for (int n = 0; n < NSP; ++n) r0[n] = sp(i, j, k, n);
    const double T = get_t_given_ey(ei, r0, P.Ru);
#pragma unroll
    for (int n = 0; n < NSP; n++) cc[n] = r0[n] / c_mech.mw[n] * 1e-6;
    for (int a = 0; a < NSP; ++a)
        for (int b = 0; b < NSP; ++b) U(a, b) = 0.0;
    production_rate(wdot, U, cc, T, P.Ru, P.Patm);
    for (int a = 0; a < NSP; ++a) {
        for (int b = 0; b < NSP; ++b) {
            const double ar = U(a, b);
            double v = (a == b ? 1.0 : 0.0);
            v -= ar * c_mech.mw[a] / c_mech.mw[b] * dt;
            U(a, b) = v;
        }
        U(a, NSP) = wdot[a] * c_mech.mw[a] * 1e6 * dt;
    }
    gauss_solve(U, drho);
    double dei = 0;
#pragma unroll
    for (int n = 0; n < NSP; ++n) {
        double v = r0[n] + drho[n];
        if (v < 0) v = 0.0;
        sp(i, j, k, n) = v;
    }
#pragma unroll
    for (int n = 0; n < NSP; ++n) dei += -c_mech.HP[n] * P.Ru / c_mech.mw[n] * drho[n];
    S(i, j, k, 4) += dei;
}

// Species clip and rescale to the mixture density, Source/EBR.cpp:341-355
__global__ void k_spec_renorm(View<const double> S, View<double> sp, CellBox B) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < B.count();
         c += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        B.cell(c, i, j, k);
        double r[NSP], rho0 = 0;
#pragma unroll
        for (int n = 0; n < NSP; ++n) {
            r[n] = sp(i, j, k, n);
            if (r[n] < 0) r[n] = 0.0;
            rho0 += r[n];
        }
        const double tmp = S(i, j, k, 0) / rho0;
#pragma unroll
        for (int n = 0; n < NSP; ++n) sp(i, j, k, n) = r[n] * tmp;
    }
}

ocfd_status configure_chem() {
    if (cudaFuncSetAttribute(k_chem_advance, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(double) * 90 * kChemThreads)) != cudaSuccess)
        return check_launch("configure_chem");
    return OCFD_OK;
}

static CellBox cellbox(const ocfd_box& bx) {
    CellBox B;
    for (int d = 0; d < 3; ++d) {
        B.lo[d] = bx.lo[d];
        B.n[d] = bx.hi[d] - bx.lo[d] + 1;
    }
    return B;
}

}  // namespace ocfd

using namespace ocfd;

extern "C" ocfd_status ocfd_chem_advance_box_f64(ocfd_context* ctx, const ocfd_array4* S,
                                                 const ocfd_array4* spec, ocfd_box bx, double dt,
                                                 void* stream) {
    if (!ctx) return fail(OCFD_BAD_ARG, "ocfd_chem_advance_box_f64: null context");
    for (int d = 0; d < 3; ++d)
        if (bx.hi[d] < bx.lo[d]) return fail(OCFD_BAD_ARG, "ocfd_chem_advance_box_f64: empty box");
    if (!covers(S, bx, 0, 5) || !covers(spec, bx, 0, NSP))
        return fail(OCFD_BAD_ARG, "ocfd_chem_advance_box_f64: S (5 comps) and spec (9 comps) must cover bx");
    if (!(dt >= 0)) return fail(OCFD_BAD_ARG, "ocfd_chem_advance_box_f64: dt must be >= 0");
    const CellBox B = cellbox(bx);
    const long long n = (long long)B.n[0] * B.n[1] * B.n[2];
    const int blocks = (int)((n + kChemThreads - 1) / kChemThreads);
    k_chem_advance<<<blocks, kChemThreads, sizeof(double) * 90 * kChemThreads, static_cast<cudaStream_t>(stream)>>>(
        view_of<double>(S), view_of<double>(spec), B, dt, ctx->parm);
    return check_launch("ocfd_chem_advance_box_f64");
}

extern "C" ocfd_status ocfd_spec_renorm_box_f64(ocfd_context* ctx, const ocfd_array4* S,
                                                const ocfd_array4* spec, ocfd_box bx, void* stream) {
    if (!ctx) return fail(OCFD_BAD_ARG, "ocfd_spec_renorm_box_f64: null context");
    for (int d = 0; d < 3; ++d)
        if (bx.hi[d] < bx.lo[d]) return fail(OCFD_BAD_ARG, "ocfd_spec_renorm_box_f64: empty box");
    if (!covers(S, bx, 0, 1) || !covers(spec, bx, 0, NSP))
        return fail(OCFD_BAD_ARG, "ocfd_spec_renorm_box_f64: S and spec must cover bx");
    const CellBox B = cellbox(bx);
    const long long n = (long long)B.n[0] * B.n[1] * B.n[2];
    long long blocks = (n + 255) / 256;
    if (blocks > (long long)ctx->num_sms * 16) blocks = (long long)ctx->num_sms * 16;
    k_spec_renorm<<<(int)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        view_of<const double>(S), view_of<double>(spec), B);
    return check_launch("ocfd_spec_renorm_box_f64");
}
