// Li-Dryer chemistry on the GPU: mechanism tables in constant memory and the
// kernels that read them (real-gas primitives, transport, multispecies RHS,
// implicit chemistry substep).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>

#include <algorithm>

#include "chem_internal.h"
#include "weno_f32.cuh"
#include "chem_physics.cuh"
#include "mlp_kernel.cuh"
#include "eb_physics.cuh"
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
    MechDerived md{};
    for (int h = 0; h < 2; ++h)
        for (int n = 0; n < NSP; ++n) {
            const double* a = h ? t.hi[n] : t.lo[n];
            md.q3[h][n] = a[2] / 3.0;
            md.q5[h][n] = a[4] / 5.0;
            md.g6[h][n] = a[2] / 6.0;
            md.g12[h][n] = a[3] / 12.0;
            md.g20[h][n] = a[4] / 20.0;
        }
    for (int a = 0; a < NSP; ++a) {
        md.inv_mw[a] = 1.0 / t.mw[a];
        for (int b = 0; b < NSP; ++b) md.wratio[a][b] = t.mw[a] / t.mw[b];
        // speciesInternalEnergy (LiDryer.H:531-614) at 250 K (low range) and 3500 K (high range)
        auto ums = [&](double T, int hi) {
            const double* c = hi ? t.hi[a] : t.lo[a];
            double u = c[0] - 1.0 + c[1] / 2.0 * T + c[2] / 3.0 * T * T + c[3] / 4.0 * T * T * T +
                       c[4] / 5.0 * T * T * T * T;
            if (hi) u += (c[5] - t.lo[a][5]) / T;
            return u;
        };
        md.umin_w[a] = ums(250.0, 0) * md.inv_mw[a];
        md.umax_w[a] = ums(3500.0, 1) * md.inv_mw[a];
    }
    if (cudaMemcpyToSymbol(c_mder, &md, sizeof(md)) != cudaSuccess) {
        cudaError_t e = cudaGetLastError();
        return fail(OCFD_LAUNCH_FAIL, std::string("mechanism upload: ") + cudaGetErrorString(e));
    }
    TransF tf{};
    for (int i = 0; i < NSP * 5; ++i) {
        tf.visc[i] = (float)t.visc[i];
        tf.cond[i] = (float)t.cond[i];
    }
    for (int i = 0; i < 45 * 5; ++i) tf.diff[i] = (float)t.diff[i];
    for (int k = 0; k < NSP; ++k) {
        tf.mw[k] = (float)t.mw[k];
        for (int j = 0; j < NSP; ++j) {
            tf.wr14[k][j] = (float)std::sqrt(std::sqrt(t.mw[j] / t.mw[k]));
            tf.den[k][j] = (float)(1.0 / std::sqrt(8.0 + 8.0 * t.mw[k] / t.mw[j]));
            tf.wratio[k][j] = (float)(t.mw[j] / t.mw[k]);
        }
    }
    if (cudaMemcpyToSymbol(c_trf, &tf, sizeof(tf)) != cudaSuccess) {
        cudaError_t e = cudaGetLastError();
        return fail(OCFD_LAUNCH_FAIL, std::string("transport upload: ") + cudaGetErrorString(e));
    }
    return OCFD_OK;
}

// One semi-implicit chemistry substep of one cell, in place: the lambda of
// EBR::chemical_advance, Source/CHEM/ChemAdvance.cpp:27-82.  u = rho, mx, my,
// mz, E (E updated), r = the 9 partial densities (updated).
__device__ __forceinline__ void chem_cell(const double* u, double& E, double* r, double dt, const DevParm& P,
                                          const SmemMat& U) {
    const double rho = dmax(u[0], P.smallr);
    const double rhoinv = 1.0 / rho;
    const double ux = u[1] * rhoinv, uy = u[2] * rhoinv, uz = u[3] * rhoinv;
    const double kineng = 0.5 * (ux * ux + uy * uy + uz * uz);
    const double ei = E - rho * kineng;
    double cc[NSP], wdot[NSP], drho[NSP];
    const double T = get_t_given_ey(ei, r, P.Ru);
#pragma unroll
    for (int n = 0; n < NSP; n++) cc[n] = r[n] * c_mder.inv_mw[n] * 1e-6;
    for (int a = 0; a < NSP; ++a)
        for (int b = 0; b < NSP; ++b) U(a, b) = 0.0;
    production_rate(wdot, U, cc, T, P.Ru, P.Patm);
    for (int a = 0; a < NSP; ++a) {
        for (int b = 0; b < NSP; ++b) {
            const double ar = U(a, b);
            double v = (a == b ? 1.0 : 0.0);
            v -= ar * c_mder.wratio[a][b] * dt;
            U(a, b) = v;
        }
        U(a, NSP) = wdot[a] * c_mech.mw[a] * 1e6 * dt;
    }
    gauss_solve(U, drho);
    double dei = 0;
#pragma unroll
    for (int n = 0; n < NSP; ++n) {
        double v = r[n] + drho[n];
        if (v < 0) v = 0.0;
        r[n] = v;
    }
#pragma unroll
    for (int n = 0; n < NSP; ++n) dei += -c_mech.HP[n] * P.Ru * c_mder.inv_mw[n] * drho[n];
    E += dei;
}

// Species clip and rescale to the mixture density of one cell (Source/EBR.cpp:341-355),
// the same arithmetic as k_spec_renorm, applied in the epilogue of a step's last
// chemistry substep (the cell's density is untouched by the chemistry)
__device__ __forceinline__ void renorm_cell(double rho, double* r) {
    double rho0 = 0;
#pragma unroll
    for (int n = 0; n < NSP; ++n) {
        if (r[n] < 0) r[n] = 0.0;
        rho0 += r[n];
    }
    const double tmp = rho / rho0;
#pragma unroll
    for (int n = 0; n < NSP; ++n) r[n] = r[n] * tmp;
}

__global__ void __launch_bounds__(kChemThreads) k_chem_advance(View<double> S, View<double> sp, CellBox B,
                                                               double dt, DevParm P, int renorm) {
    extern __shared__ double smem[];
    const SmemMat U{smem + threadIdx.x, (int)blockDim.x};
    const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (c >= B.count()) return;
    int i, j, k;
    B.cell(c, i, j, k);
    double u[5], r[NSP];
#pragma unroll
    for (int n = 0; n < 5; ++n) u[n] = S(i, j, k, n);
#pragma unroll
    for (int n = 0; n < NSP; ++n) r[n] = sp(i, j, k, n);
    double E = u[4];
    chem_cell(u, E, r, dt, P, U);
    if (renorm) renorm_cell(u[0], r);
#pragma unroll
    for (int n = 0; n < NSP; ++n) sp(i, j, k, n) = r[n];
    S(i, j, k, 4) = E;
}

// The same substep over a list of cells of a level (element offset of component
// 0 and the component stride of each cell's FAB; state then species
// components): one launch for every box, in the list's order.
// ncell is bounded by *count when given (a list filled on the device); dtc gives
// a step per cell when given.
__global__ void __launch_bounds__(kChemThreads) k_chem_advance_list(const long long* __restrict__ off,
                                                                    const long long* __restrict__ stride,
                                                                    long long ncell, const unsigned* count,
                                                                    const double* __restrict__ dtc, double* Ubuf,
                                                                    double dt, DevParm P, int renorm) {
    extern __shared__ double smem[];
    const SmemMat U{smem + threadIdx.x, (int)blockDim.x};
    const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (count && c >= (long long)*count) return;
    if (c >= ncell) return;
    if (dtc) dt = dtc[c];
    double* x = Ubuf + off[c];
    const long long ns = stride[c];
    double u[5], r[NSP];
#pragma unroll
    for (int n = 0; n < 5; ++n) u[n] = x[n * ns];
#pragma unroll
    for (int n = 0; n < NSP; ++n) r[n] = x[(5 + n) * ns];
    double E = u[4];
    chem_cell(u, E, r, dt, P, U);
    if (renorm) renorm_cell(u[0], r);
#pragma unroll
    for (int n = 0; n < NSP; ++n) x[(5 + n) * ns] = r[n];
    x[4 * ns] = E;
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
                             (int)(sizeof(double) * 90 * kChemThreads)) != cudaSuccess ||
        cudaFuncSetAttribute(k_chem_advance_list, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(double) * 90 * kChemThreads)) != cudaSuccess)
        return check_launch("configure_chem");
    return OCFD_OK;
}

ocfd_status launch_chem_advance(View<double> S, View<double> sp, const CellBox& B, double dt, const DevParm& P,
                                cudaStream_t st, bool renorm) {
    const long long n = (long long)B.n[0] * B.n[1] * B.n[2];
    const int blocks = (int)((n + kChemThreads - 1) / kChemThreads);
    k_chem_advance<<<blocks, kChemThreads, sizeof(double) * 90 * kChemThreads, st>>>(S, sp, B, dt, P, renorm ? 1 : 0);
    return check_launch("chemistry substep");
}

ocfd_status launch_chem_advance_list(const long long* off, const long long* stride, long long ncell, double* U,
                                     double dt, const DevParm& P, cudaStream_t st, const unsigned* count,
                                     const double* dtc, bool renorm) {
    if (ncell <= 0) return OCFD_OK;
    const long long blocks = (ncell + kChemThreads - 1) / kChemThreads;
    k_chem_advance_list<<<(unsigned)blocks, kChemThreads, sizeof(double) * 90 * kChemThreads, st>>>(
        off, stride, ncell, count, dtc, U, dt, P, renorm ? 1 : 0);
    return check_launch("chemistry substep (cell list)");
}

// ------------------------------------------------------------ surrogate substep
// Temperature, pressure and mass fractions of cells of a list: T from e by the
// Newton of LiDryer.H:833-888, p = CKPY (LiDryer.H:10-18)
__device__ __forceinline__ void cell_props(const double* x, long long ns, const DevParm& P, double* T, double* p,
                                           double* Y, double* rho_out, double* r) {
    const double rho = dmax(x[0], P.smallr);
    const double rhoinv = 1.0 / rho;
    const double ux = x[ns] * rhoinv, uy = x[2 * ns] * rhoinv, uz = x[3 * ns] * rhoinv;
    const double ei = x[4 * ns] - rho * (0.5 * (ux * ux + uy * uy + uz * uz));
#pragma unroll
    for (int n = 0; n < NSP; ++n) r[n] = x[(5 + n) * ns];
    *T = get_t_given_ey(ei, r, P.Ru);
    *p = ckpy(r, *T, P.Ru);
#pragma unroll
    for (int n = 0; n < NSP; ++n) Y[n] = r[n] * rhoinv;
    *rho_out = rho;
}

__global__ void k_chem_props(const long long* __restrict__ off, const long long* __restrict__ stride, long long ncell,
                             const double* __restrict__ Ubuf, double* out, DevParm P) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell;
         c += (long long)gridDim.x * blockDim.x) {
        double T, p, Y[NSP], rho, r[NSP];
        cell_props(Ubuf + off[c], stride[c], P, &T, &p, Y, &rho, r);
        out[c] = T;
        out[ncell + c] = p;
#pragma unroll
        for (int n = 0; n < NSP; ++n) out[(2 + n) * ncell + c] = Y[n];
    }
}

// Constant-pressure restoration of 0D cells at rest after a constant-volume
// substep.  A closed adiabatic system at pressure p keeps its enthalpy; the
// constant-volume substep kept e and rho, so the enthalpy of the isobaric step
// is h = e + p_target / rho with the density before the substep.  T' solves
// sum_n Y_n h_n(T') = h (Newton on the NASA-7 enthalpy with its cp), then
// rho' = p_target / (Ru T' sum_n Y_n / W_n) and rho' E' = rho' h - p_target.
// Generator of constant-pressure ignition states; no counterpart in the
// reference, whose reactor is the constant-volume cell of
// Source/CHEM/ChemAdvance.cpp:27-82.
__global__ void k_chem_isobaric(long long ncell, double* __restrict__ U, const double* __restrict__ p_target,
                                DevParm P) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell;
         c += (long long)gridDim.x * blockDim.x) {
        double T, p, Y[NSP], rho, r[NSP];
        double* x = U + c;
        cell_props(x, ncell, P, &T, &p, Y, &rho, r);
        const double pt = p_target[c];
        const double rhoinv = 1.0 / rho;
        const double ux = x[ncell] * rhoinv, uy = x[2 * ncell] * rhoinv, uz = x[3 * ncell] * rhoinv;
        const double e = x[4 * ncell] * rhoinv - 0.5 * (ux * ux + uy * uy + uz * uz);
        const double h = e + pt * rhoinv;
        double yw = 0.0;
#pragma unroll
        for (int n = 0; n < NSP; ++n) yw += Y[n] * c_mder.inv_mw[n];
        for (int it = 0; it < 50; ++it) {
            double hs[NSP];
            species_enthalpy(T, hs);
            double hm = 0.0, cp = 0.0;
            const double T2 = T * T;
#pragma unroll
            for (int n = 0; n < NSP; ++n) {
                const double* a = nasa(T, n);
                const double w = Y[n] * c_mder.inv_mw[n];
                hm += w * hs[n];
                cp += w * (a[0] + a[1] * T + a[2] * T2 + a[3] * T2 * T + a[4] * T2 * T2);
            }
            double dT = (h / P.Ru - hm) / cp;
            dT = fmin(fmax(dT, -200.0), 200.0);
            T += dT;
            if (fabs(dT) <= 1e-10 * T) break;
        }
        const double rn = pt / (P.Ru * T * yw);
        x[0] = rn;
        x[ncell] = x[2 * ncell] = x[3 * ncell] = 0.0;
        x[4 * ncell] = rn * h - pt;
#pragma unroll
        for (int n = 0; n < NSP; ++n) x[(5 + n) * ncell] = rn * Y[n];
    }
}

// H, O, N atoms of H2, O2, H2O, H, O, OH, HO2, H2O2, N2
__constant__ float c_elem[3][NSP] = {{2, 0, 2, 1, 0, 1, 1, 2, 0}, {0, 2, 1, 0, 1, 1, 2, 2, 0}, {0, 0, 0, 0, 0, 0, 0, 0, 2}};

// FP32 thermochemistry of the surrogate substep, per unit mass, built once per
// CTA from the NASA-7 tables: the network's inputs are BF16-rounded, so T and p
// only need FP32 accuracy, and the FP64 Newton of the plain substep (divisions
// by the molar masses and by 3 and 5 in every evaluation) would cost more than
// the network itself.
struct SurThermo {
    float ce[2][NSP][6];  // e_n(T) = c5 + T (c0 + T (c1 + T (c2 + T (c3 + T c4)))) [J/kg], T < 1000 K | >= 1000 K
    float iw[NSP];        // 1 / W_n
    float elem[3][NSP];   // atoms per unit mass (mol/kg) of each element
    double hw[NSP];       // d(rho e)/d(rho_n) of the chemistry update, -HP_n Ru / W_n (ChemAdvance.cpp:70-75)
};
constexpr int S_THERMO = (S_TOT + 15) / 16 * 16;
constexpr int S_SUR_TOT = S_THERMO + (int)sizeof(SurThermo);

__device__ __forceinline__ void sur_thermo_build(SurThermo& th, double Ru) {
    const int n = threadIdx.x;
    if (n >= NSP) return;
    const double rw = Ru / c_mech.mw[n];
    for (int h = 0; h < 2; ++h) {
        const double* a = h ? c_mech.hi[n] : c_mech.lo[n];
        // e/(RT) of speciesInternalEnergy (LiDryer.H:531-614) times R T / W
        th.ce[h][n][0] = (float)(rw * (a[0] - 1.0));
        th.ce[h][n][1] = (float)(rw * a[1] / 2.0);
        th.ce[h][n][2] = (float)(rw * a[2] / 3.0);
        th.ce[h][n][3] = (float)(rw * a[3] / 4.0);
        th.ce[h][n][4] = (float)(rw * a[4] / 5.0);
        th.ce[h][n][5] = (float)(h ? rw * (a[5] - c_mech.lo[n][5]) : 0.0);
    }
    th.iw[n] = (float)(1.0 / c_mech.mw[n]);
    for (int e = 0; e < 3; ++e) th.elem[e][n] = (float)(c_elem[e][n] / c_mech.mw[n]);
    th.hw[n] = -c_mech.HP[n] * Ru / c_mech.mw[n];
}

// T from the internal energy per unit mass: Newton on the mixture polynomial
// (its coefficients summed once), a fixed five iterations from 1500 K (the
// energy is close to linear in T, so the error after five is at FP32 rounding
// for 250-3500 K); T is kept inside [200, 5000] K on the way.
__device__ __forceinline__ float sur_temperature(const SurThermo& th, const float* Y, float e) {
    float lo[6], hi[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) lo[k] = hi[k] = 0.0f;
#pragma unroll
    for (int n = 0; n < NSP; ++n)
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            lo[k] = fmaf(Y[n], th.ce[0][n][k], lo[k]);
            hi[k] = fmaf(Y[n], th.ce[1][n][k], hi[k]);
        }
    float T = 1500.0f;
#pragma unroll
    for (int it = 0; it < 5; ++it) {
        const bool h = T >= 1000.0f;
        float c[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) c[k] = h ? hi[k] : lo[k];
        const float ev = fmaf(T, fmaf(T, fmaf(T, fmaf(T, fmaf(T, c[4], c[3]), c[2]), c[1]), c[0]), c[5]);
        const float cv = fmaf(T, fmaf(T, fmaf(T, fmaf(T, 5.0f * c[4], 4.0f * c[3]), 3.0f * c[2]), 2.0f * c[1]), c[0]);
        T = fminf(fmaxf(T + (e - ev) / cv, 200.0f), 5000.0f);
    }
    return T;
}

// One chemistry substep by the network for the cells of a list, 128 cells per
// tile (thread t < 128 of the first warpgroup = cell t of the tile; all MLP_G
// warpgroups share the network's epilogues): inputs (T, p, Y, log10 dt) ->
// rates of T and Y (the increments over the substep divided by dt).
// Cells whose inputs leave the training range, or whose increments break the
// species bounds or the H / O / N element balance beyond the guard's
// tolerances, are appended to the fallback list for the FP64 substep.
// Accepted cells update rho Y_n (clipped at 0) and rho E as the FP64 substep
// does (ChemAdvance.cpp:62-80).
__global__ void __launch_bounds__(128 * MLP_G) k_chem_surrogate(MlpNet net, const long long* __restrict__ off,
                                                        const long long* __restrict__ stride, long long ncell,
                                                        double* Ubuf, double dt, DevParm P, ocfd_surrogate_guard g,
                                                        long long* fb_off, long long* fb_stride, unsigned* fb_count,
                                                        unsigned long long* fb_total, unsigned* err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + S_BAR);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + S_BAR + 8);
    SurThermo& th = *reinterpret_cast<SurThermo*>(sm + S_THERMO);
    const int tid = threadIdx.x, warp = tid >> 5;
    mlp_stage_weights(net, sm);
    sur_thermo_build(th, P.Ru);
    if (tid == 0) mbar_init(bar, 1);
    if (warp == 0) {
        tmem_alloc(tslot, 128);
        tmem_relinquish();
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tbase = *tslot;
    uint32_t phase = 0;
    bool ok = true;
    const long long ntile = (ncell + 127) / 128;
    const float ldt = (float)log10(dt);
    const bool dt_in = dt >= g.dt_min && dt <= g.dt_max;
    const float Ru = (float)P.Ru, fdt = (float)dt;
    const float T_min = (float)g.T_min, T_max = (float)g.T_max, p_min = (float)g.p_min, p_max = (float)g.p_max;
    const float y_tol = (float)g.y_tol, elem_tol = (float)g.elem_tol;
    const float dy_rel = (float)g.dy_rel_max, y_floor = (float)g.y_floor;
    for (long long t = blockIdx.x; t < ntile && ok; t += gridDim.x) {
        const long long c = t * 128 + tid;
        const bool valid = tid < 128 && c < ncell;
        double* x = nullptr;
        long long ns = 0;
        double rho = 1.0, r[NSP];
        float Y[NSP], T = 0.0f, p = 1.0f;
        if (valid) {
            x = Ubuf + off[c];
            ns = stride[c];
            rho = dmax(x[0], P.smallr);
            const double rhoinv = 1.0 / rho;
            const double ux = x[ns] * rhoinv, uy = x[2 * ns] * rhoinv, uz = x[3 * ns] * rhoinv;
            const float em = (float)(x[4 * ns] * rhoinv - 0.5 * (ux * ux + uy * uy + uz * uz));
            float wsum = 0.0f;
#pragma unroll
            for (int n = 0; n < NSP; ++n) {
                r[n] = x[(5 + n) * ns];
                Y[n] = (float)(r[n] * rhoinv);
                wsum = fmaf(Y[n], th.iw[n], wsum);
            }
            T = sur_temperature(th, Y, em);
            p = (float)rho * Ru * T * wsum;
        } else {
#pragma unroll
            for (int n = 0; n < NSP; ++n) r[n] = 0.0, Y[n] = 0.0f;
        }
        // features: T, ln p, sqrt(Y), log10 dt, normalised
        float f[16];
        f[0] = (T - net.in_mu[0]) * net.in_isd[0];
        f[1] = ((valid ? logf(p) : 0.0f) - net.in_mu[1]) * net.in_isd[1];
#pragma unroll
        for (int n = 0; n < NSP; ++n) f[2 + n] = (sqrtf(fmaxf(Y[n], 0.0f)) - net.in_mu[2 + n]) * net.in_isd[2 + n];
        f[11] = (ldt - net.in_mu[11]) * net.in_isd[11];
        if (tid < 128) {
#pragma unroll
            for (int k = 0; k < 16; ++k)
                *reinterpret_cast<uint16_t*>(sm + S_A0 + kmajor_offset(tid, k, 128)) = k < MLP_IN ? bf16_bits(f[k]) : 0;
        }
        float out[16];
        ok = mlp_tile<MLP_G>(sm, tbase, bar, phase, out, nullptr, nullptr, 0);
        if (!ok || !valid) continue;
        float dY[NSP];
#pragma unroll
        for (int n = 0; n < NSP; ++n) {
            const float y = out[1 + n] * net.out_sd[1 + n] + net.out_mu[1 + n];
            const float sc = net.out_scale[1 + n];
            dY[n] = (sc > 0.0f ? copysignf(sc * expm1f(fabsf(y)), y) : y) * fdt;
        }
        bool pass = dt_in && T >= T_min && T <= T_max && p >= p_min && p <= p_max;
#pragma unroll
        for (int n = 0; n < NSP; ++n) pass = pass && Y[n] + dY[n] >= -y_tol && Y[n] + dY[n] <= 1.0f + y_tol;
        // per-output criterion: the network's error in a rate is roughly a fixed
        // fraction of the rate (its targets are logarithms of the rates), so a
        // cell whose increments change no Y by more than dy_rel of itself (or of
        // y_floor, for traces) keeps the relative error of every Y below that
        // fraction of dy_rel per substep; the rest (ignition fronts) go to FP64
        if (dy_rel > 0.0f) {
#pragma unroll
            for (int n = 0; n < NSP; ++n) pass = pass && fabsf(dY[n]) <= dy_rel * fmaxf(Y[n], y_floor);
        }
#pragma unroll
        for (int e = 0; e < 3; ++e) {
            float have = 0.0f, d = 0.0f;
#pragma unroll
            for (int n = 0; n < NSP; ++n) {
                have = fmaf(th.elem[e][n], Y[n], have);
                d = fmaf(th.elem[e][n], dY[n], d);
            }
            pass = pass && fabsf(d) <= elem_tol * have;
        }
        // accepted increments are made element-conserving: N2 is inert, and the
        // H and O imbalance is removed by the correction of least weighted norm
        // with weights |dY_n| (each increment absorbs a share of the imbalance in
        // proportion to its own size), on the increments scaled by their sum
        if (pass) {
            dY[NSP - 1] = 0.0f;
            float S = 0.0f;
#pragma unroll
            for (int n = 0; n < NSP - 1; ++n) S += fabsf(dY[n]);
            if (S > 0.0f) {
                const float iS = 1.0f / S;
                float w[NSP - 1], m00 = 0, m01 = 0, m11 = 0, r0 = 0, r1 = 0;
#pragma unroll
                for (int n = 0; n < NSP - 1; ++n) {
                    const float u = dY[n] * iS, aH = th.elem[0][n], aO = th.elem[1][n];
                    w[n] = fabsf(u) + 1e-6f;
                    m00 = fmaf(w[n] * aH, aH, m00);
                    m01 = fmaf(w[n] * aH, aO, m01);
                    m11 = fmaf(w[n] * aO, aO, m11);
                    r0 = fmaf(aH, u, r0);
                    r1 = fmaf(aO, u, r1);
                }
                const float det = m00 * m11 - m01 * m01;
                if (det > 1e-6f * m00 * m11) {
                    const float l0 = (m11 * r0 - m01 * r1) / det, l1 = (m00 * r1 - m01 * r0) / det;
#pragma unroll
                    for (int n = 0; n < NSP - 1; ++n)
                        dY[n] = S * (dY[n] * iS - w[n] * (th.elem[0][n] * l0 + th.elem[1][n] * l1));
                } else {
                    pass = false;
                }
            }
        }
        if (pass) {
            double dei = 0;
#pragma unroll
            for (int n = 0; n < NSP; ++n) {
                const double drho = rho * (double)dY[n];
                double v = r[n] + drho;
                if (v < 0) v = 0.0;
                x[(5 + n) * ns] = v;
                dei += th.hw[n] * drho;
            }
            x[4 * ns] += dei;
        } else {
            const unsigned q = atomicAdd(fb_count, 1u);
            fb_off[q] = off[c];
            fb_stride[q] = ns;
            atomicAdd(fb_total, 1ull);
        }
    }
    if (!ok && tid == 0) atomicOr(err, 1u);
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tbase, 128);
}

ocfd_status launch_chem_surrogate(const ocfd_mlp* mlp, const long long* off, const long long* stride, long long ncell,
                                  double* U, double dt, const DevParm& P, const ocfd_surrogate_guard& g,
                                  long long* fb_off, long long* fb_stride, unsigned* fb_count,
                                  unsigned long long* fb_total, unsigned* err, int sms, cudaStream_t st) {
    static bool configured = false;
    if (!configured) {
        if (cudaFuncSetAttribute(k_chem_surrogate, cudaFuncAttributeMaxDynamicSharedMemorySize, S_SUR_TOT) != cudaSuccess)
            return check_launch("surrogate attribute");
        configured = true;
    }
    if (ncell <= 0) return OCFD_OK;
    const long long ntile = (ncell + 127) / 128;
    k_chem_surrogate<<<(unsigned)std::min<long long>(ntile, sms), 128 * MLP_G, S_SUR_TOT, st>>>(
        mlp_net(mlp), off, stride, ncell, U, dt, P, g, fb_off, fb_stride, fb_count, fb_total, err);
    return check_launch("surrogate chemistry substep");
}

ocfd_status launch_spec_renorm(View<const double> S, View<double> sp, const CellBox& B, int sms, cudaStream_t st) {
    const long long n = (long long)B.n[0] * B.n[1] * B.n[2];
    long long blocks = (n + 255) / 256;
    if (blocks > (long long)sms * 16) blocks = (long long)sms * 16;
    k_spec_renorm<<<(int)blocks, 256, 0, st>>>(S, sp, B);
    return check_launch("species renormalisation");
}

// Conserved state of a resting mixture at (T, p, X): CKXTY, CKRHOY, CKUBMS as
// the reference's initial conditions use them (Exec/7_JET/prob.H:46-60).
__global__ void k_chem_state_tpx(long long n, const double* T, const double* p, const double* X, double* U,
                                 double* rhoY, double Ru) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        double x[NSP], y[NSP], r[NSP];
#pragma unroll
        for (int i = 0; i < NSP; ++i) x[i] = X[i * n + c];
        double XW = 0.0;
#pragma unroll
        for (int i = 0; i < NSP; ++i) XW += x[i] * c_mech.mw[i];
#pragma unroll
        for (int i = 0; i < NSP; ++i) y[i] = x[i] * c_mech.mw[i] / XW;
        double YOW = 0, tmp[NSP];
#pragma unroll
        for (int i = 0; i < NSP; ++i) tmp[i] = y[i] / c_mech.mw[i];
#pragma unroll
        for (int i = 0; i < NSP; ++i) YOW += tmp[i];
        const double rho = p[c] / (Ru * T[c] * YOW);
#pragma unroll
        for (int i = 0; i < NSP; ++i) r[i] = rho * y[i];
        U[c] = rho;
        U[n + c] = 0.0;
        U[2 * n + c] = 0.0;
        U[3 * n + c] = 0.0;
        U[4 * n + c] = ckubms(T[c], r, Ru);
#pragma unroll
        for (int i = 0; i < NSP; ++i) rhoY[i * n + c] = r[i];
    }
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
    return launch_chem_advance(view_of<double>(S), view_of<double>(spec), cellbox(bx), dt, ctx->parm,
                               static_cast<cudaStream_t>(stream));
}

extern "C" ocfd_status ocfd_spec_renorm_box_f64(ocfd_context* ctx, const ocfd_array4* S,
                                                const ocfd_array4* spec, ocfd_box bx, void* stream) {
    if (!ctx) return fail(OCFD_BAD_ARG, "ocfd_spec_renorm_box_f64: null context");
    for (int d = 0; d < 3; ++d)
        if (bx.hi[d] < bx.lo[d]) return fail(OCFD_BAD_ARG, "ocfd_spec_renorm_box_f64: empty box");
    if (!covers(S, bx, 0, 1) || !covers(spec, bx, 0, NSP))
        return fail(OCFD_BAD_ARG, "ocfd_spec_renorm_box_f64: S and spec must cover bx");
    return launch_spec_renorm(view_of<const double>(S), view_of<double>(spec), cellbox(bx), ctx->num_sms,
                              static_cast<cudaStream_t>(stream));
}

// =====================================================================
// Multispecies right-hand side of a regular box: replaces the kernel chain
// of EBR::compute_dSdt_multi, Source/CHEM/FlowAdvance.cpp:157-403.
//   k_chem_prims    c2prim_rgas over grow(bx, 3)        (Kernels.H:42-81)
//   k_chem_trans    mu, lambda, D over grow(bx, 1)      (FlowAdvance.cpp:188-202)
//   k_chem_faces<D> per face, in registers: Steger-Warming split of the 6
//                   stencil cells (flow with the local gamma, species by the
//                   split factor of FlowAdvance.cpp:214-242), WENO-Z of the
//                   5 + 9 components, Fick diffusion (ChemViscous.H:108-199),
//                   multispecies viscous + heat + species-enthalpy flux
//                   (ChemViscous.H:201-355)
//   k_chem_div      divop for the 5 + 9 components       (Kernels.H:84-97)
// =====================================================================
namespace ocfd {

// c2prim_rgas, Source/kernel/Kernels.H:42-81
__device__ __forceinline__ void c2prim_real(const DevParm& P, const double* u, const double* rhoi, double* q) {
    const double rho = dmax(u[0], P.smallr);
    const double rhoinv = 1.0 / rho;
    const double ux = u[1] * rhoinv, uy = u[2] * rhoinv, uz = u[3] * rhoinv;
    const double kineng = 0.5 * (ux * ux + uy * uy + uz * uz);
    const double ei = u[4] - rho * kineng;
    q[QRHO] = rho;
    q[QU] = ux;
    q[QV] = uy;
    q[QW] = uz;
    const double T = get_t_given_ey(ei, rhoi, P.Ru);
    const double p = ckpy(rhoi, T, P.Ru);
    q[QT] = T;
    q[QPRES] = p;
    const double gama = p / ei + 1.0;
    q[QGAMA] = gama;
    q[QC] = sqrt(gama * p / rho);
}

__global__ void k_chem_prims(ChemBoxArgs B, DevParm P) {
    const int g = B.qg;
    const int gx = B.hi[0] - B.lo[0] + 1 + 2 * g, gy = B.hi[1] - B.lo[1] + 1 + 2 * g,
              gz = B.hi[2] - B.lo[2] + 1 + 2 * g;
    const long long n = (long long)gx * gy * gz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        const int i = B.lo[0] - g + (int)(c % gx), j = B.lo[1] - g + (int)((c / gx) % gy),
                  k = B.lo[2] - g + (int)(c / ((long long)gx * gy));
        double u[5], r[NSP], q[8];
#pragma unroll
        for (int m = 0; m < 5; ++m) u[m] = B.S(i, j, k, m);
#pragma unroll
        for (int m = 0; m < NSP; ++m) r[m] = B.sp(i, j, k, m);
        c2prim_real(P, u, r, q);
#pragma unroll
        for (int m = 0; m < 8; ++m) B.q(i, j, k, m) = q[m];
    }
}

// mixed form: transport in FP32 (transport_f32), widened into the FP64 array
__global__ void k_chem_trans_f32(ChemBoxArgs B) {
    const int gx = B.hi[0] - B.lo[0] + 3, gy = B.hi[1] - B.lo[1] + 3, gz = B.hi[2] - B.lo[2] + 3;
    const long long n = (long long)gx * gy * gz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        const int i = B.lo[0] - 1 + (int)(c % gx), j = B.lo[1] - 1 + (int)((c / gx) % gy),
                  k = B.lo[2] - 1 + (int)(c / ((long long)gx * gy));
        const float T = d2f_bits(B.q(i, j, k, QT)), p = d2f_bits(B.q(i, j, k, QPRES));
        const float rinv = __frcp_rn(d2f_bits(B.q(i, j, k, QRHO)));
        float Y[NSP], D[NSP], mu, lam;
#pragma unroll
        for (int m = 0; m < NSP; ++m) Y[m] = d2f_bits(B.sp(i, j, k, m)) * rinv;
        transport_f32(T, p, Y, mu, lam, D);
        B.tr(i, j, k, 0) = f2d_bits(mu);
        B.tr(i, j, k, 1) = f2d_bits(lam);
#pragma unroll
        for (int m = 0; m < NSP; ++m) B.tr(i, j, k, 2 + m) = f2d_bits(D[m]);
    }
}

__global__ void k_chem_trans(ChemBoxArgs B) {
    const int gx = B.hi[0] - B.lo[0] + 3, gy = B.hi[1] - B.lo[1] + 3, gz = B.hi[2] - B.lo[2] + 3;
    const long long n = (long long)gx * gy * gz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        const int i = B.lo[0] - 1 + (int)(c % gx), j = B.lo[1] - 1 + (int)((c / gx) % gy),
                  k = B.lo[2] - 1 + (int)(c / ((long long)gx * gy));
        double Yt[NSP], Xt[NSP], D[NSP];
        const double T = B.q(i, j, k, QT), p = B.q(i, j, k, QPRES), rho = B.q(i, j, k, QRHO);
#pragma unroll
        for (int m = 0; m < NSP; ++m) Yt[m] = B.sp(i, j, k, m) / rho;
        ckytx(Yt, Xt);
        double mu, lam;
        mixture_properties(T, Xt, mu, lam);
        mix_diff_coeffs(T, p, Xt, D);
        B.tr(i, j, k, 0) = mu;
        B.tr(i, j, k, 1) = lam;
#pragma unroll
        for (int m = 0; m < NSP; ++m) B.tr(i, j, k, 2 + m) = D[m];
    }
}

// Fick diffusion of the D-face (ChemViscous.H:108-199) added to the species
// face flux fs[9]; the diffusive part is returned in fd[9].
__device__ __forceinline__ void diffusion_face(const ChemBoxArgs& B, int D, int i, int j, int k,
                                               double* fs, double* fd) {
    const int li = i - (D == 0), lj = j - (D == 1), lk = k - (D == 2);
    const double rhor = B.q(i, j, k, QRHO), rhol = B.q(li, lj, lk, QRHO);
    const double rho = 0.5 * (rhol + rhor);
#pragma unroll
    for (int n = 0; n < NSP; ++n) {
        const double Ytr = B.sp(i, j, k, n) / rhor;
        const double Ytl = B.sp(li, lj, lk, n) / rhol;
        const double di = 0.5 * (B.tr(i, j, k, 2 + n) + B.tr(li, lj, lk, 2 + n));
        const double tmp = rho * di * (Ytl - Ytr) * B.dxinv[D];
        fd[n] = tmp;
        fs[n] += tmp;
    }
}

// face-averaged mu, lambda and species-enthalpy flux (ChemViscous.H:215-231)
__device__ __forceinline__ void multi_face_props(const ChemBoxArgs& B, int D, int i, int j, int k,
                                                 const double* fd, double& muf, double& lamf,
                                                 double& hflux) {
    const int li = i - (D == 0), lj = j - (D == 1), lk = k - (D == 2);
    const double Tr = B.q(i, j, k, QT), Tl = B.q(li, lj, lk, QT);
    const double T = 0.5 * (Tl + Tr);
    muf = 0.5 * (B.tr(i, j, k, 0) + B.tr(li, lj, lk, 0));
    lamf = 0.5 * (B.tr(i, j, k, 1) + B.tr(li, lj, lk, 1));
    double h[NSP];
    species_enthalpy(T, h);
    double tmp = 0;
#pragma unroll
    for (int n = 0; n < NSP; ++n) tmp += fd[n] * h[n];
    hflux = tmp;
}

// multispecies viscous flux of a regular face (ChemViscous.H:201-355)
__device__ __forceinline__ void visc_multi_face(const DevParm& P, const ChemBoxArgs& B, int D, int i,
                                                int j, int k, double* f, double muf, double lamf,
                                                double hflux) {
    const int li = i - (D == 0), lj = j - (D == 1), lk = k - (D == 2);
    const double Tr = B.q(i, j, k, QT), Tl = B.q(li, lj, lk, QT);
    const double dT = (Tr - Tl) * B.dxinv[D];
    double g[3][3];
#pragma unroll
    for (int m = 0; m < 3; ++m) g[m][D] = (B.q(i, j, k, QU + m) - B.q(li, lj, lk, QU + m)) * B.dxinv[D];
#pragma unroll
    for (int t = 0; t < 3; ++t) {
        if (t == D) continue;
        const int ti = t == 0, tj = t == 1, tk = t == 2;
        g[D][t] = (B.q(i + ti, j + tj, k + tk, QU + D) + B.q(li + ti, lj + tj, lk + tk, QU + D) -
                   B.q(i - ti, j - tj, k - tk, QU + D) - B.q(li - ti, lj - tj, lk - tk, QU + D)) *
                  (0.25 * B.dxinv[t]);
        g[t][t] = (B.q(i + ti, j + tj, k + tk, QU + t) + B.q(li + ti, lj + tj, lk + tk, QU + t) -
                   B.q(i - ti, j - tj, k - tk, QU + t) - B.q(li - ti, lj - tj, lk - tk, QU + t)) *
                  (0.25 * B.dxinv[t]);
    }
    const double divu = g[0][0] + g[1][1] + g[2][2];
    double tau[3];
#pragma unroll
    for (int m = 0; m < 3; ++m)
        tau[m] = (m == D) ? muf * (2.0 * g[D][D] - P.twoThirds * divu) : muf * (g[m][D] + g[D][m]);
#pragma unroll
    for (int m = 0; m < 3; ++m) f[1 + m] += -tau[m];
    f[4] += -0.5 * ((B.q(i, j, k, QU) + B.q(li, lj, lk, QU)) * tau[0] +
                    (B.q(i, j, k, QV) + B.q(li, lj, lk, QV)) * tau[1] +
                    (B.q(i, j, k, QW) + B.q(li, lj, lk, QW)) * tau[2]) -
            lamf * dT - hflux;
}

// Convective face fluxes in FP32 (the mixed form): the stencil's primitives and
// partial densities narrowed on the integer pipes, Steger-Warming split and the
// split factors of the species in FP32, WENO-Z on normalised stencils
// (weno_f32.cuh), widened back to FP64.
template <int D>
__device__ __forceinline__ void chem_conv_f32(const ChemBoxArgs& B, int i, int j, int k, double* f, double* fs) {
    const int di = D == 0, dj = D == 1, dk = D == 2;
    float fp[6][5], fm[6][5], t1[6], tp[6], tm[6];
#pragma unroll
    for (int s = 0; s < 6; ++s) {
        const int ci = i + (s - 3) * di, cj = j + (s - 3) * dj, ck = k + (s - 3) * dk;
        const float d = d2f_bits(B.q(ci, cj, ck, QRHO)), u = d2f_bits(B.q(ci, cj, ck, QU)),
                    v = d2f_bits(B.q(ci, cj, ck, QV)), w = d2f_bits(B.q(ci, cj, ck, QW)),
                    cs = d2f_bits(B.q(ci, cj, ck, QC)), gamma = d2f_bits(B.q(ci, cj, ck, QGAMA));
        const float tmp1 = __frcp_rn(2.0f * gamma);
        const float tmp2 = 2.0f * (gamma - 1.0f);
        const float tmp3 = __fdividef(3.0f - gamma, 2.0f * (gamma - 1.0f));
        sw_split<D, float>(d, u, v, w, cs, tmp1, tmp2, tmp3, gamma - 1.0f, fp[s], fm[s]);
        const float un = D == 0 ? u : (D == 1 ? v : w);
        const float E1 = un, E2 = un - cs, E3 = un + cs;
        const float E1P = (E1 + fabsf(E1)) * 0.5f, E2P = (E2 + fabsf(E2)) * 0.5f, E3P = (E3 + fabsf(E3)) * 0.5f;
        t1[s] = tmp1;
        tp[s] = tmp2 * E1P + E2P + E3P;
        tm[s] = tmp2 * (E1 - E1P) + (E2 - E2P) + (E3 - E3P);
    }
#pragma unroll
    for (int n = 0; n < 5; ++n)
        f[n] = f2d_bits(wenoz_pm_f(fp[0][n], fp[1][n], fp[2][n], fp[3][n], fp[4][n], fm[5][n], fm[4][n],
                                   fm[3][n], fm[2][n], fm[1][n]));
#pragma unroll
    for (int n = 0; n < NSP; ++n) {
        float a[6], b[6];
#pragma unroll
        for (int s = 0; s < 6; ++s) {
            const float tmp0 = d2f_bits(B.sp(i + (s - 3) * di, j + (s - 3) * dj, k + (s - 3) * dk, n)) * t1[s];
            a[s] = tmp0 * tp[s];
            b[s] = tmp0 * tm[s];
        }
        fs[n] = f2d_bits(wenoz_pm_f(a[0], a[1], a[2], a[3], a[4], b[5], b[4], b[3], b[2], b[1]));
    }
}

template <int D, bool F32>
__global__ void __launch_bounds__(128) k_chem_faces(ChemBoxArgs B, DevParm P) {
    const int fx = B.hi[0] - B.lo[0] + 1 + (D == 0), fy = B.hi[1] - B.lo[1] + 1 + (D == 1),
              fz = B.hi[2] - B.lo[2] + 1 + (D == 2);
    const long long nf = (long long)fx * fy * fz;
    const int di = D == 0, dj = D == 1, dk = D == 2;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < nf;
         c += (long long)gridDim.x * blockDim.x) {
        const int i = B.lo[0] + (int)(c % fx), j = B.lo[1] + (int)((c / fx) % fy),
                  k = B.lo[2] + (int)(c / ((long long)fx * fy));
        double f[5], fs[NSP];
        if (F32) {
            chem_conv_f32<D>(B, i, j, k, f, fs);
        } else {
        // split of the stencil cells i-3 .. i+2 along D; s = 0..5
        double fp[6][5], fm[6][5], t1[6], tp[6], tm[6];
#pragma unroll
        for (int s = 0; s < 6; ++s) {
            const int ci = i + (s - 3) * di, cj = j + (s - 3) * dj, ck = k + (s - 3) * dk;
            const double d = B.q(ci, cj, ck, QRHO), u = B.q(ci, cj, ck, QU), v = B.q(ci, cj, ck, QV),
                         w = B.q(ci, cj, ck, QW), cs = B.q(ci, cj, ck, QC), gamma = B.q(ci, cj, ck, QGAMA);
            const double tmp1 = 1.0 / (2.0 * gamma);
            const double tmp2 = 2.0 * (gamma - 1.0);
            const double tmp3 = (3.0 - gamma) / (2.0 * (gamma - 1.0));
            sw_split<D>(d, u, v, w, cs, tmp1, tmp2, tmp3, gamma - 1, fp[s], fm[s]);
            const double un = D == 0 ? u : (D == 1 ? v : w);
            const double E1 = un, E2 = un - cs, E3 = un + cs;
            const double E1P = (E1 + fabs(E1)) * 0.5, E2P = (E2 + fabs(E2)) * 0.5, E3P = (E3 + fabs(E3)) * 0.5;
            const double E1M = E1 - E1P, E2M = E2 - E2P, E3M = E3 - E3P;
            t1[s] = tmp1;
            tp[s] = tmp2 * E1P + E2P + E3P;
            tm[s] = tmp2 * E1M + E2M + E3M;
        }
#pragma unroll
        for (int n = 0; n < 5; ++n)
            f[n] = wenoz_1rcp(fp[0][n], fp[1][n], fp[2][n], fp[3][n], fp[4][n]) +
                   wenoz_1rcp(fm[5][n], fm[4][n], fm[3][n], fm[2][n], fm[1][n]);
#pragma unroll
        for (int n = 0; n < NSP; ++n) {
            double a[6], b[6];
#pragma unroll
            for (int s = 0; s < 6; ++s) {
                const double tmp0 = B.sp(i + (s - 3) * di, j + (s - 3) * dj, k + (s - 3) * dk, n) * t1[s];
                a[s] = tmp0 * tp[s];
                b[s] = tmp0 * tm[s];
            }
            fs[n] = wenoz_1rcp(a[0], a[1], a[2], a[3], a[4]) + wenoz_1rcp(b[5], b[4], b[3], b[2], b[1]);
        }
        }
        if (B.visc) {
            double fd[NSP], muf, lamf, hflux;
            diffusion_face(B, D, i, j, k, fs, fd);
            multi_face_props(B, D, i, j, k, fd, muf, lamf, hflux);
            visc_multi_face(P, B, D, i, j, k, f, muf, lamf, hflux);
        }
#pragma unroll
        for (int n = 0; n < 5; ++n) B.flux[D](i, j, k, n) = f[n];
#pragma unroll
        for (int n = 0; n < NSP; ++n) B.fluxs[D](i, j, k, n) = fs[n];
    }
}

__global__ void k_chem_div(ChemBoxArgs B) {
    const int nx = B.hi[0] - B.lo[0] + 1, ny = B.hi[1] - B.lo[1] + 1, nz = B.hi[2] - B.lo[2] + 1;
    const long long n = (long long)nx * ny * nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        const int i = B.lo[0] + (int)(c % nx), j = B.lo[1] + (int)((c / nx) % ny),
                  k = B.lo[2] + (int)(c / ((long long)nx * ny));
#pragma unroll
        for (int m = 0; m < 5; ++m)
            B.dsdt(i, j, k, m) = B.dxinv[0] * (B.flux[0](i, j, k, m) - B.flux[0](i + 1, j, k, m)) +
                                 B.dxinv[1] * (B.flux[1](i, j, k, m) - B.flux[1](i, j + 1, k, m)) +
                                 B.dxinv[2] * (B.flux[2](i, j, k, m) - B.flux[2](i, j, k + 1, m));
#pragma unroll
        for (int m = 0; m < NSP; ++m)
            B.dsdts(i, j, k, m) = B.dxinv[0] * (B.fluxs[0](i, j, k, m) - B.fluxs[0](i + 1, j, k, m)) +
                                  B.dxinv[1] * (B.fluxs[1](i, j, k, m) - B.fluxs[1](i, j + 1, k, m)) +
                                  B.dxinv[2] * (B.fluxs[2](i, j, k, m) - B.fluxs[2](i, j, k + 1, m));
    }
}

// ---- cut-cell multispecies box, Source/CHEM/FlowAdvanceBox.cpp:105-499 ----
// Van Leer species flux of one face, FlowAdvanceBox.cpp:166-223
__device__ __forceinline__ void vanleer_spec(const double* ql, const double* qr, const double* rl,
                                             const double* rr, int D, double* fs) {
    double fp[NSP], fm[NSP];
#pragma unroll
    for (int n = 0; n < NSP; ++n) {
        fp[n] = 0;
        fm[n] = 0;
    }
    const double ul = ql[QU + D], ur = qr[QU + D];
    const double cL = ql[QC], cR = qr[QC];
    const double ML = ul / cL, MR = ur / cR, UL = ul, UR = ur;
    if (ML >= 1.0) {
#pragma unroll
        for (int n = 0; n < NSP; ++n) fp[n] = rl[n] * UL;
    } else if (fabs(ML) < 1.0) {
        const double Mp = 0.250 * (1.0 + ML) * (1.0 + ML);
#pragma unroll
        for (int n = 0; n < NSP; ++n) fp[n] = rl[n] * cL * Mp;
    }
    if (fabs(MR) < 1.0) {
        const double Mm = -0.250 * (MR - 1.0) * (MR - 1.0);
#pragma unroll
        for (int n = 0; n < NSP; ++n) fm[n] = rr[n] * cR * Mm;
    } else if (MR <= -1.0) {
#pragma unroll
        for (int n = 0; n < NSP; ++n) fm[n] = rr[n] * UR;
    }
#pragma unroll
    for (int n = 0; n < NSP; ++n) fs[n] = fp[n] + fm[n];
}

template <int D>
__global__ void __launch_bounds__(128) k_chem_eb_faces(ChemBoxArgs B, DevParm P) {
    const int fx = B.hi[0] - B.lo[0] + 1 + (D == 0), fy = B.hi[1] - B.lo[1] + 1 + (D == 1),
              fz = B.hi[2] - B.lo[2] + 1 + (D == 2);
    const long long nf = (long long)fx * fy * fz;
    const int di = D == 0, dj = D == 1, dk = D == 2;
    const View<const double> q{B.q.p, B.q.js, B.q.ks, B.q.ns, B.q.b0, B.q.b1, B.q.b2};
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < nf;
         c += (long long)gridDim.x * blockDim.x) {
        const int i = B.lo[0] + (int)(c % fx), j = B.lo[1] + (int)((c / fx) % fy),
                  k = B.lo[2] + (int)(c / ((long long)fx * fy));
        const uint32_t f = B.flag(i, j, k);
        double ql[8], qr[8], rl[NSP], rr[NSP], flx[5], fs[NSP];
#pragma unroll
        for (int m = 0; m < 8; ++m)
            eb_recon(f, D, q(i - 2 * di, j - 2 * dj, k - 2 * dk, m), q(i - di, j - dj, k - dk, m),
                     q(i, j, k, m), q(i + di, j + dj, k + dk, m), ql[m], qr[m]);
#pragma unroll
        for (int m = 0; m < NSP; ++m)
            eb_recon(f, D, B.sp(i - 2 * di, j - 2 * dj, k - 2 * dk, m), B.sp(i - di, j - dj, k - dk, m),
                     B.sp(i, j, k, m), B.sp(i + di, j + dj, k + dk, m), rl[m], rr[m]);
        vanleer<double>(P.smallp, 0.5 * (ql[QGAMA] + qr[QGAMA]), ql, qr, D, flx);
        vanleer_spec(ql, qr, rl, rr, D, fs);
        if (B.visc) {
            double fd[NSP], muf, lamf, hflux;
            diffusion_face(B, D, i, j, k, fs, fd);
            multi_face_props(B, D, i, j, k, fd, muf, lamf, hflux);
            eb_visc_face(P, q, B.flag, D, i, j, k, B.dxinv, flx, 1, true, muf, lamf, hflux);
        }
#pragma unroll
        for (int n = 0; n < 5; ++n) B.flux[D](i, j, k, n) = flx[n];
#pragma unroll
        for (int n = 0; n < NSP; ++n) B.fluxs[D](i, j, k, n) = fs[n];
    }
}

// species divergence of a cut box (FlowAdvanceBox.cpp:407-460), negated; the
// flow dSdt of a cut multispecies box is left zero as the reference leaves it
// (its divc -> dSdt copy is commented out, FlowAdvanceBox.cpp:500-523)
__global__ void k_chem_eb_div(ChemBoxArgs B) {
    const int nx = B.hi[0] - B.lo[0] + 1, ny = B.hi[1] - B.lo[1] + 1, nz = B.hi[2] - B.lo[2] + 1;
    const long long n = (long long)nx * ny * nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
         c += (long long)gridDim.x * blockDim.x) {
        const int i = B.lo[0] + (int)(c % nx), j = B.lo[1] + (int)((c / nx) % ny),
                  k = B.lo[2] + (int)(c / ((long long)nx * ny));
#pragma unroll
        for (int m = 0; m < 5; ++m) B.dsdt(i, j, k, m) = 0.0;
        const uint32_t f = B.flag(i, j, k);
        const double tmp = B.dxinv[0] / B.vfrac(i, j, k);
        double out[NSP];
        if (eb_covered(f)) {
#pragma unroll
            for (int m = 0; m < NSP; ++m) out[m] = 0.0;
        } else if (eb_regular(f)) {
#pragma unroll
            for (int m = 0; m < NSP; ++m)
                out[m] = B.dxinv[0] * (B.fluxs[0](i + 1, j, k, m) - B.fluxs[0](i, j, k, m)) +
                         B.dxinv[1] * (B.fluxs[1](i, j + 1, k, m) - B.fluxs[1](i, j, k, m)) +
                         B.dxinv[2] * (B.fluxs[2](i, j, k + 1, m) - B.fluxs[2](i, j, k, m));
        } else {
            const double axm = B.ap[0](i, j, k), axp = B.ap[0](i + 1, j, k);
            const double aym = B.ap[1](i, j, k), ayp = B.ap[1](i, j + 1, k);
            const double azm = B.ap[2](i, j, k), azp = B.ap[2](i, j, k + 1);
#pragma unroll
            for (int m = 0; m < NSP; ++m)
                out[m] = tmp * (axp * B.fluxs[0](i + 1, j, k, m) - axm * B.fluxs[0](i, j, k, m) +
                                ayp * B.fluxs[1](i, j + 1, k, m) - aym * B.fluxs[1](i, j, k, m) +
                                azp * B.fluxs[2](i, j, k + 1, m) - azm * B.fluxs[2](i, j, k, m));
            if (B.visc) {
                const double apnorm = sqrt((axm - axp) * (axm - axp) + (aym - ayp) * (aym - ayp) +
                                           (azm - azp) * (azm - azp));
                const double un = B.q(i, j, k, QU) * (axm - axp) + B.q(i, j, k, QV) * (aym - ayp) +
                                  B.q(i, j, k, QW) * (azm - azp);
                const double lambda0 = fabs(un) + B.q(i, j, k, QC) * apnorm;
#pragma unroll
                for (int m = 0; m < NSP; ++m) {
                    const double sn = B.sp(i, j, k, m);
                    const double fpw = 0.5 * (sn * un + lambda0 * sn);
                    const double fmw = -0.5 * (sn * un + lambda0 * sn);
                    out[m] += (fpw + fmw) * tmp;
                }
            }
        }
#pragma unroll
        for (int m = 0; m < NSP; ++m) B.dsdts(i, j, k, m) = out[m] * -1.0;
    }
}

static int chem_blocks(long long n, int threads, int sms) {
    long long b = (n + threads - 1) / threads;
    long long cap = (long long)sms * 64;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

size_t chem_rhs_scratch_doubles(const ocfd_box& bx) {
    const int n[3] = {bx.hi[0] - bx.lo[0] + 1, bx.hi[1] - bx.lo[1] + 1, bx.hi[2] - bx.lo[2] + 1};
    const long long qcells = (long long)(n[0] + 6) * (n[1] + 6) * (n[2] + 6);
    const long long tcells = (long long)(n[0] + 2) * (n[1] + 2) * (n[2] + 2);
    long long f = 0;
    for (int d = 0; d < 3; ++d) f += (long long)(n[0] + (d == 0)) * (n[1] + (d == 1)) * (n[2] + (d == 2));
    return (size_t)(8 * qcells + 11 * tcells + (5 + NSP) * f);
}

void chem_rhs_args(ChemBoxArgs& B, View<const double> S, View<const double> sp, View<double> dsdt,
                   View<double> dsdts, const ocfd_box& bx, const double dxinv[3], bool visc, double* scr) {
    B = ChemBoxArgs{};
    const int n[3] = {bx.hi[0] - bx.lo[0] + 1, bx.hi[1] - bx.lo[1] + 1, bx.hi[2] - bx.lo[2] + 1};
    const int g = 3;
    const long long qcells = (long long)(n[0] + 2 * g) * (n[1] + 2 * g) * (n[2] + 2 * g);
    const long long tcells = (long long)(n[0] + 2) * (n[1] + 2) * (n[2] + 2);
    B.S = S;
    B.sp = sp;
    B.dsdt = dsdt;
    B.dsdts = dsdts;
    for (int d = 0; d < 3; ++d) {
        B.lo[d] = bx.lo[d];
        B.hi[d] = bx.hi[d];
        B.dxinv[d] = dxinv[d];
    }
    B.q = View<double>{scr, n[0] + 2 * g, (long long)(n[0] + 2 * g) * (n[1] + 2 * g), qcells, bx.lo[0] - g,
                       bx.lo[1] - g, bx.lo[2] - g};
    B.qg = g;
    scr += 8 * qcells;
    B.tr = View<double>{scr, n[0] + 2, (long long)(n[0] + 2) * (n[1] + 2), tcells, bx.lo[0] - 1, bx.lo[1] - 1,
                        bx.lo[2] - 1};
    scr += 11 * tcells;
    for (int d = 0; d < 3; ++d) {
        const int sx = n[0] + (d == 0), sy = n[1] + (d == 1);
        const long long fc = (long long)sx * sy * (n[2] + (d == 2));
        B.flux[d] = View<double>{scr, sx, (long long)sx * sy, fc, bx.lo[0], bx.lo[1], bx.lo[2]};
        scr += 5 * fc;
        B.fluxs[d] = View<double>{scr, sx, (long long)sx * sy, fc, bx.lo[0], bx.lo[1], bx.lo[2]};
        scr += NSP * fc;
    }
    B.visc = visc ? 1 : 0;
}

// the kernel chain of one regular box (regular branch of compute_dSdt_multi)
ocfd_status launch_chem_rhs(const ChemBoxArgs& B, const DevParm& P, int sms, cudaStream_t st) {
    const int n[3] = {B.hi[0] - B.lo[0] + 1, B.hi[1] - B.lo[1] + 1, B.hi[2] - B.lo[2] + 1};
    const long long qcells = (long long)(n[0] + 2 * B.qg) * (n[1] + 2 * B.qg) * (n[2] + 2 * B.qg);
    const long long tcells = (long long)(n[0] + 2) * (n[1] + 2) * (n[2] + 2);
    k_chem_prims<<<chem_blocks(qcells, 128, sms), 128, 0, st>>>(B, P);
    if (B.visc) {
        if (B.f32) k_chem_trans_f32<<<chem_blocks(tcells, 128, sms), 128, 0, st>>>(B);
        else k_chem_trans<<<chem_blocks(tcells, 128, sms), 128, 0, st>>>(B);
    }
    const long long nfx = (long long)(n[0] + 1) * n[1] * n[2], nfy = (long long)n[0] * (n[1] + 1) * n[2],
                    nfz = (long long)n[0] * n[1] * (n[2] + 1);
    if (B.f32) {
        k_chem_faces<0, true><<<chem_blocks(nfx, 128, sms), 128, 0, st>>>(B, P);
        k_chem_faces<1, true><<<chem_blocks(nfy, 128, sms), 128, 0, st>>>(B, P);
        k_chem_faces<2, true><<<chem_blocks(nfz, 128, sms), 128, 0, st>>>(B, P);
    } else {
        k_chem_faces<0, false><<<chem_blocks(nfx, 128, sms), 128, 0, st>>>(B, P);
        k_chem_faces<1, false><<<chem_blocks(nfy, 128, sms), 128, 0, st>>>(B, P);
        k_chem_faces<2, false><<<chem_blocks(nfz, 128, sms), 128, 0, st>>>(B, P);
    }
    k_chem_div<<<chem_blocks((long long)n[0] * n[1] * n[2], 256, sms), 256, 0, st>>>(B);
    return check_launch("multispecies RHS");
}

// The cut-cell multispecies chain of one box (ebchem_compute_dSdt_box,
// Source/CHEM/FlowAdvanceBox.cpp:16-525): primitives over grow(bx, 2),
// transport, the three directions' MUSCL + Van Leer faces with the species
// fluxes, the cut-cell divergence; FP64 in every form.
ocfd_status launch_chem_eb_rhs(const ChemBoxArgs& B, const DevParm& P, int sms, cudaStream_t st) {
    const int n[3] = {B.hi[0] - B.lo[0] + 1, B.hi[1] - B.lo[1] + 1, B.hi[2] - B.lo[2] + 1};
    const long long qcells = (long long)(n[0] + 2 * B.qg) * (n[1] + 2 * B.qg) * (n[2] + 2 * B.qg);
    const long long tcells = (long long)(n[0] + 2) * (n[1] + 2) * (n[2] + 2);
    k_chem_prims<<<chem_blocks(qcells, 128, sms), 128, 0, st>>>(B, P);
    if (B.visc) k_chem_trans<<<chem_blocks(tcells, 128, sms), 128, 0, st>>>(B);
    k_chem_eb_faces<0><<<chem_blocks((long long)(n[0] + 1) * n[1] * n[2], 128, sms), 128, 0, st>>>(B, P);
    k_chem_eb_faces<1><<<chem_blocks((long long)n[0] * (n[1] + 1) * n[2], 128, sms), 128, 0, st>>>(B, P);
    k_chem_eb_faces<2><<<chem_blocks((long long)n[0] * n[1] * (n[2] + 1), 128, sms), 128, 0, st>>>(B, P);
    k_chem_eb_div<<<chem_blocks((long long)n[0] * n[1] * n[2], 256, sms), 256, 0, st>>>(B);
    return check_launch("multispecies cut-cell RHS");
}

void chem_args_as_cut(ChemBoxArgs& B, View<const uint32_t> flag, View<const double> vfrac,
                      const View<const double> ap[3]) {
    // the primitives over grow(bx, 2) at the start of the same scratch (the
    // grow(bx, 3) block of the regular layout holds them)
    const int g = 2;
    const int n[3] = {B.hi[0] - B.lo[0] + 1, B.hi[1] - B.lo[1] + 1, B.hi[2] - B.lo[2] + 1};
    const long long qcells = (long long)(n[0] + 2 * g) * (n[1] + 2 * g) * (n[2] + 2 * g);
    B.q = View<double>{B.q.p, n[0] + 2 * g, (long long)(n[0] + 2 * g) * (n[1] + 2 * g), qcells, B.lo[0] - g,
                       B.lo[1] - g, B.lo[2] - g};
    B.qg = g;
    B.eb = 1;
    B.f32 = 0;
    B.flag = flag;
    B.vfrac = vfrac;
    for (int d = 0; d < 3; ++d) B.ap[d] = ap[d];
}

// Shared set-up of the regular and cut-cell multispecies box calls.
static ocfd_status chem_box_setup(ocfd_context* ctx, const ocfd_array4* S, const ocfd_array4* spec,
                                  const ocfd_array4* dSdt, const ocfd_array4* dSdt_spec,
                                  const ocfd_array4* flux, const ocfd_array4* flux_spec,
                                  const ocfd_box& bx, const double dxinv[3], unsigned flags,
                                  int grow, const char* who, ChemBoxArgs& B) {
    if (!ctx || !dxinv) return fail(OCFD_BAD_ARG, std::string(who) + ": null argument");
    for (int d = 0; d < 3; ++d)
        if (bx.hi[d] < bx.lo[d]) return fail(OCFD_BAD_ARG, std::string(who) + ": empty box");
    if (!covers(S, bx, grow, 5) || !covers(spec, bx, grow, NSP))
        return fail(OCFD_BAD_ARG, std::string(who) + ": S / spec must cover grow(bx," + std::to_string(grow) + ")");
    if (!covers(dSdt, bx, 0, 5) || !covers(dSdt_spec, bx, 0, NSP))
        return fail(OCFD_BAD_ARG, std::string(who) + ": dSdt / dSdt_spec must cover bx");
    for (int d = 0; d < 3; ++d) {
        if (flux && !covers(&flux[d], bx, 0, 5, d)) return fail(OCFD_BAD_ARG, std::string(who) + ": flux[d]");
        if (flux_spec && !covers(&flux_spec[d], bx, 0, NSP, d))
            return fail(OCFD_BAD_ARG, std::string(who) + ": flux_spec[d]");
    }
    const int n[3] = {bx.hi[0] - bx.lo[0] + 1, bx.hi[1] - bx.lo[1] + 1, bx.hi[2] - bx.lo[2] + 1};
    // primitive halo: WENO needs 3 cells (regular boxes), MUSCL 2 (cut boxes)
    const int g = grow >= 3 ? 3 : 2;
    const long long qcells = (long long)(n[0] + 2 * g) * (n[1] + 2 * g) * (n[2] + 2 * g);
    const long long tcells = (long long)(n[0] + 2) * (n[1] + 2) * (n[2] + 2);
    long long fcells[3];
    for (int d = 0; d < 3; ++d) fcells[d] = (long long)(n[0] + (d == 0)) * (n[1] + (d == 1)) * (n[2] + (d == 2));
    size_t need = sizeof(double) * (8 * qcells + 11 * tcells);
    if (!flux) need += sizeof(double) * 5 * (fcells[0] + fcells[1] + fcells[2]);
    if (!flux_spec) need += sizeof(double) * NSP * (fcells[0] + fcells[1] + fcells[2]);
    double* scr = static_cast<double*>(scratch(ctx, need));
    if (!scr) return fail(OCFD_OUT_OF_MEMORY, std::string(who) + ": scratch");
    B.S = view_of<const double>(S);
    B.sp = view_of<const double>(spec);
    B.dsdt = view_of<double>(dSdt);
    B.dsdts = view_of<double>(dSdt_spec);
    for (int d = 0; d < 3; ++d) {
        B.lo[d] = bx.lo[d];
        B.hi[d] = bx.hi[d];
        B.dxinv[d] = dxinv[d];
    }
    B.q = View<double>{scr, n[0] + 2 * g, (long long)(n[0] + 2 * g) * (n[1] + 2 * g), qcells,
                       bx.lo[0] - g, bx.lo[1] - g, bx.lo[2] - g};
    B.qg = g;
    scr += 8 * qcells;
    B.tr = View<double>{scr, n[0] + 2, (long long)(n[0] + 2) * (n[1] + 2), tcells, bx.lo[0] - 1,
                        bx.lo[1] - 1, bx.lo[2] - 1};
    scr += 11 * tcells;
    for (int d = 0; d < 3; ++d) {
        const int sx = n[0] + (d == 0), sy = n[1] + (d == 1);
        if (flux) {
            B.flux[d] = view_of<double>(&flux[d]);
        } else {
            B.flux[d] = View<double>{scr, sx, (long long)sx * sy, fcells[d], bx.lo[0], bx.lo[1], bx.lo[2]};
            scr += 5 * fcells[d];
        }
        if (flux_spec) {
            B.fluxs[d] = view_of<double>(&flux_spec[d]);
        } else {
            B.fluxs[d] = View<double>{scr, sx, (long long)sx * sy, fcells[d], bx.lo[0], bx.lo[1], bx.lo[2]};
            scr += NSP * fcells[d];
        }
    }
    B.visc = (flags & OCFD_VISC) != 0;
    return OCFD_OK;
}

}  // namespace ocfd

extern "C" ocfd_status ocfd_rhs_chem_box_f64(ocfd_context* ctx, const ocfd_array4* S,
                                             const ocfd_array4* spec, const ocfd_array4* dSdt,
                                             const ocfd_array4* dSdt_spec, const ocfd_array4* flux,
                                             const ocfd_array4* flux_spec, ocfd_box bx,
                                             const double dxinv[3], unsigned flags, void* stream) {
    using namespace ocfd;
    if (flags & ~(unsigned)OCFD_VISC) return fail(OCFD_BAD_ARG, "ocfd_rhs_chem_box_f64: unsupported flags");
    ChemBoxArgs B{};
    ocfd_status s = chem_box_setup(ctx, S, spec, dSdt, dSdt_spec, flux, flux_spec, bx, dxinv, flags, 3,
                                   "ocfd_rhs_chem_box_f64", B);
    if (s != OCFD_OK) return s;
    return launch_chem_rhs(B, ctx->parm, ctx->num_sms, static_cast<cudaStream_t>(stream));
}

extern "C" ocfd_status ocfd_chem_state_tpx(ocfd_context* ctx, int64_t n, const double* T, const double* p,
                                           const double* X, double* U, double* rhoY, void* stream) {
    using namespace ocfd;
    if (!ctx || n < 0 || (n > 0 && (!T || !p || !X || !U || !rhoY)))
        return fail(OCFD_BAD_ARG, "ocfd_chem_state_tpx: bad arguments");
    if (n == 0) return OCFD_OK;
    long long blocks = (n + 255) / 256;
    if (blocks > (long long)ctx->num_sms * 16) blocks = (long long)ctx->num_sms * 16;
    k_chem_state_tpx<<<(int)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(n, T, p, X, U, rhoY, ctx->parm.Ru);
    return check_launch("ocfd_chem_state_tpx");
}

extern "C" ocfd_status ocfd_rhs_chem_eb_box_f64(ocfd_context* ctx, const ocfd_array4* S,
                                                const ocfd_array4* spec, const ocfd_array4* dSdt,
                                                const ocfd_array4* dSdt_spec, const ocfd_array4* flux,
                                                const ocfd_array4* flux_spec, const ocfd_flag4* flag,
                                                const ocfd_array4* vfrac, const ocfd_array4* apx,
                                                const ocfd_array4* apy, const ocfd_array4* apz,
                                                const ocfd_array4* const* fc, const ocfd_array4* bcent,
                                                ocfd_box bx, const double dxinv[3], unsigned flags,
                                                void* stream) {
    using namespace ocfd;
    (void)fc;
    (void)bcent;
    if (flags & ~(unsigned)OCFD_VISC) return fail(OCFD_BAD_ARG, "ocfd_rhs_chem_eb_box_f64: unsupported flags");
    if (!covers_flag(flag, bx, 1)) return fail(OCFD_BAD_ARG, "ocfd_rhs_chem_eb_box_f64: flag must cover grow(bx,1)");
    if (!covers(vfrac, bx, 0, 1)) return fail(OCFD_BAD_ARG, "ocfd_rhs_chem_eb_box_f64: vfrac must cover bx");
    const ocfd_array4* ap[3] = {apx, apy, apz};
    for (int d = 0; d < 3; ++d)
        if (!covers(ap[d], bx, 0, 1, d)) return fail(OCFD_BAD_ARG, "ocfd_rhs_chem_eb_box_f64: area fractions");
    ChemBoxArgs B{};
    ocfd_status s = chem_box_setup(ctx, S, spec, dSdt, dSdt_spec, flux, flux_spec, bx, dxinv, flags, 2,
                                   "ocfd_rhs_chem_eb_box_f64", B);
    if (s != OCFD_OK) return s;
    B.eb = 1;
    B.flag = view_of_flag(flag);
    B.vfrac = view_of<const double>(vfrac);
    for (int d = 0; d < 3; ++d) B.ap[d] = view_of<const double>(ap[d]);
    return launch_chem_eb_rhs(B, ctx->parm, ctx->num_sms, static_cast<cudaStream_t>(stream));
}

// ------------------------------------------------------------ 0D cells
namespace ocfd {
__global__ void k_iota_cells(long long* off, long long* stride, long long n) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        off[c] = c;
        stride[c] = n;
    }
}

struct CellList {
    long long* off = nullptr;
    long long* stride = nullptr;
    ~CellList() {
        cudaFree(off);
        cudaFree(stride);
    }
    bool make(long long n, int sms, cudaStream_t st) {
        if (cudaMalloc(&off, sizeof(long long) * n) != cudaSuccess ||
            cudaMalloc(&stride, sizeof(long long) * n) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        long long b = (n + 255) / 256;
        if (b > (long long)sms * 16) b = (long long)sms * 16;
        k_iota_cells<<<(int)b, 256, 0, st>>>(off, stride, n);
        return true;
    }
};
}  // namespace ocfd

extern "C" ocfd_status ocfd_chem_cells_advance(ocfd_context* ctx, int64_t n, double* U, const double* dt_cells,
                                               double dt, void* stream) {
    using namespace ocfd;
    if (!ctx || n <= 0 || !U) return fail(OCFD_BAD_ARG, "ocfd_chem_cells_advance");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CellList L;
    if (!L.make(n, ctx->num_sms, st)) return fail(OCFD_OUT_OF_MEMORY, "ocfd_chem_cells_advance");
    ocfd_status s = launch_chem_advance_list(L.off, L.stride, n, U, dt, ctx->parm, st, nullptr, dt_cells);
    if (cudaStreamSynchronize(st) != cudaSuccess) return check_launch("ocfd_chem_cells_advance");
    return s;
}

extern "C" ocfd_status ocfd_chem_cells_props(ocfd_context* ctx, int64_t n, const double* U, double* out,
                                             void* stream) {
    using namespace ocfd;
    if (!ctx || n <= 0 || !U || !out) return fail(OCFD_BAD_ARG, "ocfd_chem_cells_props");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CellList L;
    if (!L.make(n, ctx->num_sms, st)) return fail(OCFD_OUT_OF_MEMORY, "ocfd_chem_cells_props");
    long long b = (n + 127) / 128;
    if (b > (long long)ctx->num_sms * 32) b = (long long)ctx->num_sms * 32;
    k_chem_props<<<(int)b, 128, 0, st>>>(L.off, L.stride, n, U, out, ctx->parm);
    ocfd_status s = check_launch("ocfd_chem_cells_props");
    if (cudaStreamSynchronize(st) != cudaSuccess) return check_launch("ocfd_chem_cells_props");
    return s;
}

extern "C" ocfd_status ocfd_chem_cells_isobaric(ocfd_context* ctx, int64_t n, double* U, const double* p_target,
                                                void* stream) {
    using namespace ocfd;
    if (!ctx || n <= 0 || !U || !p_target) return fail(OCFD_BAD_ARG, "ocfd_chem_cells_isobaric");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    long long b = (n + 127) / 128;
    if (b > (long long)ctx->num_sms * 32) b = (long long)ctx->num_sms * 32;
    k_chem_isobaric<<<(int)b, 128, 0, st>>>(n, U, p_target, ctx->parm);
    ocfd_status s = check_launch("ocfd_chem_cells_isobaric");
    if (cudaStreamSynchronize(st) != cudaSuccess) return check_launch("ocfd_chem_cells_isobaric");
    return s;
}

extern "C" ocfd_status ocfd_chem_cells_surrogate(ocfd_context* ctx, ocfd_mlp* mlp, const ocfd_surrogate_guard* g,
                                                 int64_t n, double* U, double dt, int64_t* fallbacks,
                                                 void* stream) {
    using namespace ocfd;
    if (!ctx || !mlp || !g || n <= 0 || !U) return fail(OCFD_BAD_ARG, "ocfd_chem_cells_surrogate");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CellList L, F;
    unsigned* cnt = nullptr;
    unsigned long long* tot = nullptr;
    if (!L.make(n, ctx->num_sms, st) || !F.make(n, ctx->num_sms, st) || cudaMalloc(&cnt, sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc(&tot, sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(cnt);
        return fail(OCFD_OUT_OF_MEMORY, "ocfd_chem_cells_surrogate");
    }
    cudaMemsetAsync(cnt, 0, sizeof(unsigned), st);
    cudaMemsetAsync(tot, 0, sizeof(unsigned long long), st);
    cudaMemsetAsync(ctx->d_error, 0, sizeof(uint32_t), st);
    ocfd_status s = launch_chem_surrogate(mlp, L.off, L.stride, n, U, dt, ctx->parm, *g, F.off, F.stride, cnt, tot,
                                          ctx->d_error, ctx->num_sms, st);
    if (s == OCFD_OK) s = launch_chem_advance_list(F.off, F.stride, n, U, dt, ctx->parm, st, cnt, nullptr);
    unsigned long long h = 0;
    uint32_t e = 0;
    if (cudaMemcpyAsync(&h, tot, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&e, ctx->d_error, sizeof(e), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        s = check_launch("ocfd_chem_cells_surrogate");
    cudaFree(cnt);
    cudaFree(tot);
    if (s == OCFD_OK && e) s = fail(OCFD_TIMEOUT, "ocfd_chem_cells_surrogate: a tensor-core completion wait ran out");
    if (fallbacks) *fallbacks = (int64_t)h;
    return s;
}
