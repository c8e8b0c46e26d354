// Box-level CPU driver around OpenCFD-AMR's own point kernels.
//
// The reference's kernel headers (Source/kernel/*.H, Source/EB/*.H,
// Source/CHEM/*.H) and Source/Constants.cpp are compiled UNMODIFIED against the
// project-written AMReX stand-ins in oracle/shim.  This file only supplies the
// loops, in the order the reference's box drivers launch them:
//   regular box : Source/Advance.cpp:231-329
//   cut-cell box: Source/EB/AdvanceBox.cpp:78-214
//   CHEM box    : Source/CHEM/FlowAdvance.cpp:157-403
//   CHEM cut box: Source/CHEM/FlowAdvanceBox.cpp:105-499 (its lambdas restated)
//   chemistry   : Source/CHEM/ChemAdvance.cpp:27-82 (its lambda restated)
//   CFL dt      : Source/Advance.cpp:10-59 (ebr_estdt restated; it lives in a .cpp)
// Built twice by oracle/Makefile: once plain (NPRIM=7) and once with -DCHEM.
// Test infrastructure only: the result is the reference arithmetic that the
// restated oracle and the CUDA kernels are checked against.
//
// Array convention of every entry point (relative indices, box interior
// [0,nx)x[0,ny)x[0,nz), NG=4 ghosts):
//   cell arrays over the grown box, i fastest, component slowest, begin -NG;
//   dSdt over the interior; x-face arrays over (nx+1) x ny x nz, begin 0 (same for y, z).
#include <AMReX_FArrayBox.H>
#include <IndexDefines.H>
#include <Constants.H>
#include <Kernels.H>
#include <FluxSplit.H>
#include <Reconstruction.H>
#include <Diffusion.H>
#include <EBkernels.H>
#include <EBdiffusion.H>
#ifdef CHEM
#include <LiDryer.H>
#include <ChemViscous.H>
#endif

#include <limits>

using amrex::Real;
using amrex::Array4;
using amrex::Dim3;

namespace {
constexpr int NG = 4;

struct Geo {
    int nx, ny, nz;
    long long gx() const { return nx + 2 * NG; }
    long long gy() const { return ny + 2 * NG; }
    long long gz() const { return nz + 2 * NG; }
};

template <class T>
Array4<T> grown(T* p, Geo const& g, int nc) {
    return Array4<T>(p, g.gx(), g.gx() * g.gy(), g.gx() * g.gy() * g.gz(),
                     Dim3{-NG, -NG, -NG}, Dim3{g.nx + NG, g.ny + NG, g.nz + NG}, nc);
}
template <class T>
Array4<T> interior(T* p, Geo const& g, int nc) {
    long long sx = g.nx, sy = g.ny, sz = g.nz;
    return Array4<T>(p, sx, sx * sy, sx * sy * sz, Dim3{0, 0, 0}, Dim3{g.nx, g.ny, g.nz}, nc);
}
template <class T>
Array4<T> faces(T* p, Geo const& g, int dir, int nc) {
    long long sx = g.nx + (dir == 0), sy = g.ny + (dir == 1), sz = g.nz + (dir == 2);
    return Array4<T>(p, sx, sx * sy, sx * sy * sz, Dim3{0, 0, 0},
                     Dim3{(int)sx, (int)sy, (int)sz}, nc);
}
// all-nodal box surroundingNodes(bx)
template <class T>
Array4<T> nodal(T* p, Geo const& g, int nc) {
    long long sx = g.nx + 1, sy = g.ny + 1, sz = g.nz + 1;
    return Array4<T>(p, sx, sx * sy, sx * sy * sz, Dim3{0, 0, 0},
                     Dim3{(int)sx, (int)sy, (int)sz}, nc);
}

template <class F>
void for_grown(Geo const& g, F&& f) {
    for (int k = -NG; k < g.nz + NG; ++k)
        for (int j = -NG; j < g.ny + NG; ++j)
            for (int i = -NG; i < g.nx + NG; ++i) f(i, j, k);
}
template <class F>
void for_box(Geo const& g, F&& f) {
    for (int k = 0; k < g.nz; ++k)
        for (int j = 0; j < g.ny; ++j)
            for (int i = 0; i < g.nx; ++i) f(i, j, k);
}
template <class F>
void for_faces(Geo const& g, int dir, F&& f) {
    for (int k = 0; k < g.nz + (dir == 2); ++k)
        for (int j = 0; j < g.ny + (dir == 1); ++j)
            for (int i = 0; i < g.nx + (dir == 0); ++i) f(i, j, k);
}

Parm& the_parm() {
    static Parm* p = [] {
        Parm* q = new Parm{};
        q->Initialize();
        return q;
    }();
    return *p;
}

}  // namespace

extern "C" {

// Parm scalars after Parm::Initialize (Source/Constants.cpp:7-12), in
// declaration order of Source/Constants.H:9-30.
void ocfdr_parm_scalars(double* out) {
    Parm const& p = the_parm();
    double v[16] = {p.eos_gamma, p.eos_m, p.Patm, p.cv, p.cp, p.Ru, p.Rg, p.kOverMu,
                    p.Pr, p.C_s, p.T_s, p.smallr, p.smallp, p.eps, p.twoThirds, p.oneSix};
    for (int i = 0; i < 16; ++i) out[i] = v[i];
}

int ocfdr_nprim() { return NPRIM; }

// c2prim over the grown box (Source/kernel/Kernels.H:13-40 / 42-81 with CHEM).
void ocfdr_c2prim(const double* S, const double* spec, int nx, int ny, int nz, double* q) {
    Geo g{nx, ny, nz};
    auto s = grown<const double>(S, g, NCONS);
    auto qa = grown<double>(q, g, NPRIM);
    Parm const& parm = the_parm();
#ifdef CHEM
    auto sp = grown<const double>(spec, g, NSPECS);
    for_grown(g, [&](int i, int j, int k) { c2prim_rgas(i, j, k, s, sp, qa, parm); });
#else
    (void)spec;
    for_grown(g, [&](int i, int j, int k) { c2prim(i, j, k, s, qa, parm); });
#endif
}

#ifndef CHEM
// Regular (uncut) box RHS, Source/Advance.cpp:231-329.
void ocfdr_rhs_regular(const double* S, int nx, int ny, int nz, const double* dxinv_in,
                       int do_visc, double* dSdt, double* fx, double* fy, double* fz) {
    Geo g{nx, ny, nz};
    Parm const& parm = the_parm();
    amrex::GpuArray<Real, 3> dxinv{{dxinv_in[0], dxinv_in[1], dxinv_in[2]}};
    long long ng = g.gx() * g.gy() * g.gz();
    std::vector<double> qv(ng * NPRIM), fpv(ng * NCONS), fmv(ng * NCONS);
    auto s = grown<const double>(S, g, NCONS);
    auto q = grown<double>(qv.data(), g, NPRIM);
    auto fp = grown<double>(fpv.data(), g, NCONS);
    auto fm = grown<double>(fmv.data(), g, NCONS);
    double* fl[3] = {fx, fy, fz};
    for (int d = 0; d < 3; ++d) {
        auto f = faces<double>(fl[d], g, d, NCONS);
        long long n = (long long)(nx + (d == 0)) * (ny + (d == 1)) * (nz + (d == 2)) * NCONS;
        std::fill(f.p, f.p + n, 0.0);
    }
    for_grown(g, [&](int i, int j, int k) { c2prim(i, j, k, s, q, parm); });
    for (int d = 0; d < 3; ++d) {
        auto f = faces<double>(fl[d], g, d, NCONS);
        for_grown(g, [&](int i, int j, int k) {
            if (d == 0) flux_split_x(i, j, k, fp, fm, q, s, parm);
            if (d == 1) flux_split_y(i, j, k, fp, fm, q, s, parm);
            if (d == 2) flux_split_z(i, j, k, fp, fm, q, s, parm);
        });
        for_faces(g, d, [&](int i, int j, int k) {
            for (int n = 0; n < NCONS; ++n) {
                if (d == 0) reconstruction_x(i, j, k, n, fp, fm, f, parm);
                if (d == 1) reconstruction_y(i, j, k, n, fp, fm, f, parm);
                if (d == 2) reconstruction_z(i, j, k, n, fp, fm, f, parm);
            }
        });
        if (do_visc) {
            for_faces(g, d, [&](int i, int j, int k) {
                if (d == 0) compute_visc_x(i, j, k, q, f, dxinv, parm);
                if (d == 1) compute_visc_y(i, j, k, q, f, dxinv, parm);
                if (d == 2) compute_visc_z(i, j, k, q, f, dxinv, parm);
            });
        }
    }
    auto dsdt = interior<double>(dSdt, g, NCONS);
    auto fxa = faces<const double>(fx, g, 0, NCONS);
    auto fya = faces<const double>(fy, g, 1, NCONS);
    auto fza = faces<const double>(fz, g, 2, NCONS);
    for_box(g, [&](int i, int j, int k) {
        for (int n = 0; n < NCONS; ++n) divop(i, j, k, n, dsdt, fxa, fya, fza, dxinv);
    });
}
#endif

// Cut-cell box RHS, Source/EB/AdvanceBox.cpp:78-214 (plain) and the flow part of
// Source/CHEM/FlowAdvanceBox.cpp.  flag/vfrac over the grown box; apx/apy/apz
// over the face boxes of the interior.
#ifndef CHEM
void ocfdr_rhs_eb(const double* S, const uint32_t* flag_in, const double* vfrac_in,
                  const double* apx_in, const double* apy_in, const double* apz_in, int nx,
                  int ny, int nz, const double* dxinv_in, int do_visc, int do_redistribute,
                  double* dSdt, double* fx, double* fy, double* fz) {
    Geo g{nx, ny, nz};
    Parm const& parm = the_parm();
    amrex::GpuArray<Real, 3> dxinv{{dxinv_in[0], dxinv_in[1], dxinv_in[2]}};
    amrex::GpuArray<Real, 3> weights{{0., 1., 0.5}};
    long long ng = g.gx() * g.gy() * g.gz();
    long long nn = (long long)(nx + 1) * (ny + 1) * (nz + 1);
    std::vector<double> qv(ng * NPRIM), qlv(nn * NPRIM, 1.0), qrv(nn * NPRIM, 1.0),
        divcv((long long)nx * ny * nz * NCONS, 0.0);
    auto s = grown<const double>(S, g, NCONS);
    auto q = grown<double>(qv.data(), g, NPRIM);
    auto ql = nodal<double>(qlv.data(), g, NPRIM);
    auto qr = nodal<double>(qrv.data(), g, NPRIM);
    auto flag = grown<const amrex::EBCellFlag>(reinterpret_cast<const amrex::EBCellFlag*>(flag_in), g, 1);
    auto vfrac = grown<const double>(vfrac_in, g, 1);
    Array4<const double> ap[3] = {faces<const double>(apx_in, g, 0, 1),
                                  faces<const double>(apy_in, g, 1, 1),
                                  faces<const double>(apz_in, g, 2, 1)};
    Array4<const double> none;
    auto dsdt = interior<double>(dSdt, g, NCONS);
    auto divc = interior<double>(divcv.data(), g, NCONS);
    double* fl[3] = {fx, fy, fz};
    for (int d = 0; d < 3; ++d) {
        long long n = (long long)(nx + (d == 0)) * (ny + (d == 1)) * (nz + (d == 2)) * NCONS;
        std::fill(fl[d], fl[d] + n, 0.0);
    }
    for_box(g, [&](int i, int j, int k) {
        for (int n = 0; n < NCONS; ++n) { dsdt(i, j, k, n) = 0.0; divc(i, j, k, n) = 0.0; }
    });
    for_grown(g, [&](int i, int j, int k) { c2prim(i, j, k, s, q, parm); });
    for (int d = 0; d < 3; ++d) {
        auto f = faces<double>(fl[d], g, d, NCONS);
        for_faces(g, d, [&](int i, int j, int k) {
            for (int n = 0; n < NPRIM; ++n) {
                if (d == 0) eb_recon_x(i, j, k, n, vfrac, ql, qr, q, flag, parm);
                if (d == 1) eb_recon_y(i, j, k, n, vfrac, ql, qr, q, flag, parm);
                if (d == 2) eb_recon_z(i, j, k, n, vfrac, ql, qr, q, flag, parm);
            }
        });
        for_faces(g, d, [&](int i, int j, int k) { eb_flux(i, j, k, ql, qr, f, d, parm); });
        if (do_visc) {
            for_faces(g, d, [&](int i, int j, int k) {
                if (d == 0) eb_compute_visc_x(i, j, k, q, f, flag, dxinv, weights, parm);
                if (d == 1) eb_compute_visc_y(i, j, k, q, f, flag, dxinv, weights, parm);
                if (d == 2) eb_compute_visc_z(i, j, k, q, f, flag, dxinv, weights, parm);
            });
        }
    }
    auto fxa = faces<double>(fx, g, 0, NCONS);
    auto fya = faces<double>(fy, g, 1, NCONS);
    auto fza = faces<double>(fz, g, 2, NCONS);
    for_box(g, [&](int i, int j, int k) {
        if (do_visc)
            eb_compute_div_visc(i, j, k, q, divc, fxa, fya, fza, flag, vfrac, none, ap[0], ap[1],
                                ap[2], none, none, none, dxinv, parm);
        else
            eb_compute_div(i, j, k, q, divc, fxa, fya, fza, flag, vfrac, none, ap[0], ap[1], ap[2],
                           none, none, none, dxinv, parm);
    });
    if (do_redistribute) {
        amrex::IntVect lo{{0, 0, 0}}, hi{{nx - 1, ny - 1, nz - 1}};
        for_box(g, [&](int i, int j, int k) {
            if (vfrac(i, j, k) < 0.5 && vfrac(i, j, k) > 0.0) {
                flux_redist(i, j, k, lo, hi, dsdt, divc, flag, vfrac);
            } else {
                for (int n = 0; n < NCONS; ++n) dsdt(i, j, k, n) = divc(i, j, k, n);
            }
        });
    } else {
        for_box(g, [&](int i, int j, int k) {
            for (int n = 0; n < NCONS; ++n) dsdt(i, j, k, n) = divc(i, j, k, n);
        });
    }
}
#endif

// CFL time step of one box interior, Source/Advance.cpp:10-59 (CHEM: fixed 1e-8).
double ocfdr_estdt(const double* S, int nx, int ny, int nz, const double* dx) {
    Geo g{nx, ny, nz};
    Parm const& parm = the_parm();
    auto state = grown<const double>(S, g, NCONS);
    Real dt = std::numeric_limits<Real>::max();
    for_box(g, [&](int i, int j, int k) {
        Real rho = state(i, j, k, URHO);
        Real mx = state(i, j, k, UMX);
        Real my = state(i, j, k, UMY);
        Real mz = state(i, j, k, UMZ);
        Real E = state(i, j, k, UEDEN);
        Real rhoinv = Real(1.0) / amrex::max(rho, parm.smallr);
        Real vx = mx * rhoinv;
        Real vy = my * rhoinv;
        Real vz = mz * rhoinv;
        Real p = amrex::max((parm.eos_gamma - Real(1.0)) *
                                (E - Real(0.5) * rho * (vx * vx + vy * vy + vz * vz)),
                            parm.smallp);
        Real cs = std::sqrt(parm.eos_gamma * p * rhoinv);
        Real dtx = dx[0] / (std::abs(vx) + cs);
        Real dty = dx[1] / (std::abs(vy) + cs);
        Real dtz = dx[2] / (std::abs(vz) + cs);
        dt = amrex::min(dt, amrex::min(dtx, amrex::min(dty, dtz)));
    });
#ifdef CHEM
    dt = 1e-8;
#endif
    return dt;
}

#ifdef CHEM
// ---------------------------------------------------------------- chemistry
int ocfdr_nspecs() { return NSPECS; }

void ocfdr_chem_tables(double* mw, double* lo, double* hi, double* hp, double* a0,
                       double* visc, double* cond, double* diff) {
    Parm const& p = the_parm();
    const double* los[NSPECS] = {p.H2_lo, p.O2_lo, p.H2O_lo, p.H_lo, p.O_lo,
                                 p.OH_lo, p.HO2_lo, p.H2O2_lo, p.N2_lo};
    const double* his[NSPECS] = {p.H2_hi, p.O2_hi, p.H2O_hi, p.H_hi, p.O_hi,
                                 p.OH_hi, p.HO2_hi, p.H2O2_hi, p.N2_hi};
    for (int n = 0; n < NSPECS; ++n) {
        mw[n] = p.mw[n];
        hp[n] = p.HP[n];
        a0[n] = p.A0[n];
        for (int c = 0; c < 7; ++c) { lo[n * 7 + c] = los[n][c]; hi[n * 7 + c] = his[n][c]; }
    }
    for (int i = 0; i < NSPECS * 5; ++i) { visc[i] = p.visccoeff[i]; cond[i] = p.conductcoeff[i]; }
    for (int i = 0; i < 45 * 5; ++i) diff[i] = p.diffcoeff[i];
}

void ocfdr_ckxty(const double* x, double* y) { CKXTY(x, y, the_parm()); }
void ocfdr_ckytx(const double* y, double* x) { CKYTX(y, x, the_parm()); }
double ocfdr_ckrhoy(double P, double T, const double* y) {
    double rho; CKRHOY(P, T, y, rho, the_parm()); return rho;
}
double ocfdr_ckubms(double T, const double* rhoi) {
    double e; CKUBMS(T, rhoi, e, the_parm()); return e;
}
double ocfdr_ckpy(const double* rhoi, double T) {
    double p; CKPY(rhoi, T, p, the_parm()); return p;
}
double ocfdr_get_t_given_ey(double e, const double* rhoi_in) {
    double rhoi[NSPECS]; for (int n = 0; n < NSPECS; ++n) rhoi[n] = rhoi_in[n];
    double T; GET_T_GIVEN_EY(e, rhoi, T, the_parm()); return T;
}
void ocfdr_production_rate(const double* c, double T, double* wdot, double* arate) {
    Real A[NSPECS][NSPECS];
    vproductionRate(wdot, A, c, T, the_parm());
    for (int i = 0; i < NSPECS; ++i) for (int j = 0; j < NSPECS; ++j) arate[i * NSPECS + j] = A[i][j];
}
void ocfdr_gauss(const double* a, const double* b, double* x) {
    Real A[NSPECS][NSPECS];
    for (int i = 0; i < NSPECS; ++i) for (int j = 0; j < NSPECS; ++j) A[i][j] = a[i * NSPECS + j];
    gauss(x, A, b);
}
void ocfdr_mixture_properties(double T, const double* X, double* mu, double* lambda) {
    mixtureProperties(T, X, *mu, *lambda, the_parm());
}
void ocfdr_mix_diff_coeffs(double T, double p, const double* X, double* D) {
    Array4<double> Da(D, 1, 1, 1, Dim3{0, 0, 0}, Dim3{1, 1, 1}, NSPECS);
    getMixDiffCoeffsMass(0, 0, 0, T, p, X, Da, the_parm());
}
void ocfdr_species_enthalpy(double T, double* h) { speciesEnthalpy(T, h, the_parm()); }

// One semi-implicit chemistry substep over ncell cells, in place.  S holds the
// 5 conserved components with stride `cstride` between components, spec the 9
// partial densities with the same stride.  Restates the lambda of
// Source/CHEM/ChemAdvance.cpp:27-82.
void ocfdr_chem_advance(double* S, double* spec, long long ncell, long long cstride, double dt) {
    Parm const& parm = the_parm();
    const Parm* lparm = &parm;
    for (long long c = 0; c < ncell; ++c) {
        auto sf = [&](int n) -> double& { return S[c + n * cstride]; };
        auto rh = [&](int n) -> double& { return spec[c + n * cstride]; };
        Real T, ei;
        Real dei = 0;
        Real rhoi_0[NSPECS], wdot[NSPECS];
        Real cc[NSPECS], Arate[NSPECS][NSPECS], A1[NSPECS][NSPECS], rhoi_1[NSPECS], drho[NSPECS];
        Real rho = amrex::max(sf(URHO), lparm->smallr);
        Real rhoinv = Real(1.0) / rho;
        Real ux = sf(UMX) * rhoinv;
        Real uy = sf(UMY) * rhoinv;
        Real uz = sf(UMZ) * rhoinv;
        Real kineng = Real(0.5) * (ux * ux + uy * uy + uz * uz);
        ei = sf(UEDEN) - rho * kineng;
        for (int n = 0; n < NSPECS; ++n) rhoi_0[n] = rh(n);
        GET_T_GIVEN_EY(ei, rhoi_0, T, *lparm);
        for (int n = 0; n < NSPECS; n++) cc[n] = rhoi_0[n] / lparm->mw[n] * 1e-6;
        vproductionRate(wdot, Arate, cc, T, *lparm);
        for (int i = 0; i < NSPECS; ++i) {
            for (int j = 0; j < NSPECS; ++j) {
                A1[i][j] = (i == j ? 1.0 : 0.0);
                A1[i][j] -= Arate[i][j] * lparm->mw[i] / lparm->mw[j] * dt;
            }
        }
        for (int n = 0; n < NSPECS; ++n) rhoi_1[n] = wdot[n] * lparm->mw[n] * 1e6 * dt;
        gauss(drho, A1, rhoi_1);
        for (int n = 0; n < NSPECS; ++n) {
            rh(n) += drho[n];
            if (rh(n) < 0) rh(n) = Real(0.0);
        }
        for (int n = 0; n < NSPECS; ++n) dei += -lparm->HP[n] * lparm->Ru / lparm->mw[n] * drho[n];
        sf(UEDEN) += dei;
    }
}

// Species split of Source/CHEM/FlowAdvance.cpp:214-242 for direction d.
static void spec_split(Geo const& g, int d, Array4<double> const& q, Array4<const double> const& rhoi,
                       Array4<double> const& fp_spec, Array4<double> const& fm_spec) {
    const int qn = d == 0 ? QU : (d == 1 ? QV : QW);
    for_grown(g, [&](int i, int j, int k) {
        Real un = q(i, j, k, qn);
        Real c = q(i, j, k, QC);
        Real gamma = q(i, j, k, QGAMA);
        Real E1 = un;
        Real E2 = un - c;
        Real E3 = un + c;
        Real E1P = (E1 + amrex::Math::abs(E1)) * Real(0.5);
        Real E2P = (E2 + amrex::Math::abs(E2)) * Real(0.5);
        Real E3P = (E3 + amrex::Math::abs(E3)) * Real(0.5);
        Real E1M = E1 - E1P;
        Real E2M = E2 - E2P;
        Real E3M = E3 - E3P;
        Real tmp1 = Real(1.0) / (Real(2.0) * gamma);
        Real tmp2 = Real(2.0) * (gamma - Real(1.0));
        Real tmp2_p = tmp2 * E1P + E2P + E3P;
        Real tmp2_m = tmp2 * E1M + E2M + E3M;
        for (int n = 0; n < NSPECS; ++n) {
            Real tmp0 = rhoi(i, j, k, n) * tmp1;
            fp_spec(i, j, k, n) = tmp0 * tmp2_p;
            fm_spec(i, j, k, n) = tmp0 * tmp2_m;
        }
    });
}

// Transport properties over the grown box, Source/CHEM/FlowAdvance.cpp:188-202.
static void transport(Geo const& g, Array4<double> const& q, Array4<const double> const& rhoi,
                      Array4<double> const& mu, Array4<double> const& lambda,
                      Array4<double> const& D) {
    Parm const& parm = the_parm();
    for_grown(g, [&](int i, int j, int k) {
        Real Yt[NSPECS], Xt[NSPECS];
        Real T = q(i, j, k, QT);
        Real p = q(i, j, k, QPRES);
        for (int n = 0; n < NSPECS; ++n) Yt[n] = rhoi(i, j, k, n) / q(i, j, k, QRHO);
        CKYTX(Yt, Xt, parm);
        mixtureProperties(T, Xt, mu(i, j, k), lambda(i, j, k), parm);
        getMixDiffCoeffsMass(i, j, k, T, p, Xt, D, parm);
    });
}

// Transport property values over the grown box (mu, lambda, D[9]) for tests.
void ocfdr_transport(const double* S, const double* spec, int nx, int ny, int nz, double* mu,
                     double* lambda, double* D) {
    Geo g{nx, ny, nz};
    long long ng = g.gx() * g.gy() * g.gz();
    std::vector<double> qv(ng * NPRIM);
    auto q = grown<double>(qv.data(), g, NPRIM);
    auto s = grown<const double>(S, g, NCONS);
    auto rhoi = grown<const double>(spec, g, NSPECS);
    for_grown(g, [&](int i, int j, int k) { c2prim_rgas(i, j, k, s, rhoi, q, the_parm()); });
    transport(g, q, rhoi, grown<double>(mu, g, 1), grown<double>(lambda, g, 1),
              grown<double>(D, g, NSPECS));
}

// Regular-box multispecies RHS, Source/CHEM/FlowAdvance.cpp:157-403.
void ocfdr_rhs_chem(const double* S, const double* spec, int nx, int ny, int nz,
                    const double* dxinv_in, int do_visc, double* dSdt, double* dSdt_spec,
                    double* fx, double* fy, double* fz, double* fxs, double* fys, double* fzs,
                    double* fxd, double* fyd, double* fzd) {
    Geo g{nx, ny, nz};
    Parm const& parm = the_parm();
    amrex::GpuArray<Real, 3> dxinv{{dxinv_in[0], dxinv_in[1], dxinv_in[2]}};
    long long ng = g.gx() * g.gy() * g.gz();
    std::vector<double> qv(ng * NPRIM), fpv(ng * NCONS), fmv(ng * NCONS), fpsv(ng * NSPECS),
        fmsv(ng * NSPECS), muv(ng), lamv(ng), Dv(ng * NSPECS);
    auto s = grown<const double>(S, g, NCONS);
    auto rhoi = grown<const double>(spec, g, NSPECS);
    auto q = grown<double>(qv.data(), g, NPRIM);
    auto fp = grown<double>(fpv.data(), g, NCONS);
    auto fm = grown<double>(fmv.data(), g, NCONS);
    auto fps = grown<double>(fpsv.data(), g, NSPECS);
    auto fms = grown<double>(fmsv.data(), g, NSPECS);
    auto mu = grown<double>(muv.data(), g, 1);
    auto lambda = grown<double>(lamv.data(), g, 1);
    auto D = grown<double>(Dv.data(), g, NSPECS);
    double* fl[3] = {fx, fy, fz};
    double* fls[3] = {fxs, fys, fzs};
    double* fld[3] = {fxd, fyd, fzd};
    for (int d = 0; d < 3; ++d) {
        long long n = (long long)(nx + (d == 0)) * (ny + (d == 1)) * (nz + (d == 2));
        std::fill(fl[d], fl[d] + n * NCONS, 0.0);
        std::fill(fls[d], fls[d] + n * NSPECS, 0.0);
        if (do_visc) std::fill(fld[d], fld[d] + n * NSPECS, 0.0);
    }
    for_grown(g, [&](int i, int j, int k) { c2prim_rgas(i, j, k, s, rhoi, q, parm); });
    if (do_visc) transport(g, q, rhoi, mu, lambda, D);
    for (int d = 0; d < 3; ++d) {
        auto f = faces<double>(fl[d], g, d, NCONS);
        auto fs = faces<double>(fls[d], g, d, NSPECS);
        for_grown(g, [&](int i, int j, int k) {
            if (d == 0) flux_split_x(i, j, k, fp, fm, q, s, parm);
            if (d == 1) flux_split_y(i, j, k, fp, fm, q, s, parm);
            if (d == 2) flux_split_z(i, j, k, fp, fm, q, s, parm);
        });
        spec_split(g, d, q, rhoi, fps, fms);
        for_faces(g, d, [&](int i, int j, int k) {
            for (int n = 0; n < NCONS; ++n) {
                if (d == 0) reconstruction_x(i, j, k, n, fp, fm, f, parm);
                if (d == 1) reconstruction_y(i, j, k, n, fp, fm, f, parm);
                if (d == 2) reconstruction_z(i, j, k, n, fp, fm, f, parm);
            }
        });
        for_faces(g, d, [&](int i, int j, int k) {
            for (int n = 0; n < NSPECS; ++n) {
                if (d == 0) reconstruction_x(i, j, k, n, fps, fms, fs, parm);
                if (d == 1) reconstruction_y(i, j, k, n, fps, fms, fs, parm);
                if (d == 2) reconstruction_z(i, j, k, n, fps, fms, fs, parm);
            }
        });
        if (do_visc) {
            auto fd = faces<double>(fld[d], g, d, NSPECS);
            for_faces(g, d, [&](int i, int j, int k) {
                if (d == 0) diffusion_x(i, j, k, q, rhoi, D, fs, fd, dxinv);
                if (d == 1) diffusion_y(i, j, k, q, rhoi, D, fs, fd, dxinv);
                if (d == 2) diffusion_z(i, j, k, q, rhoi, D, fs, fd, dxinv);
            });
            for_faces(g, d, [&](int i, int j, int k) {
                if (d == 0) compute_visc_x_multi(i, j, k, q, rhoi, lambda, mu, f, fd, dxinv, parm);
                if (d == 1) compute_visc_y_multi(i, j, k, q, rhoi, lambda, mu, f, fd, dxinv, parm);
                if (d == 2) compute_visc_z_multi(i, j, k, q, rhoi, lambda, mu, f, fd, dxinv, parm);
            });
        }
    }
    auto dsdt = interior<double>(dSdt, g, NCONS);
    auto dsdts = interior<double>(dSdt_spec, g, NSPECS);
    auto fxa = faces<const double>(fx, g, 0, NCONS);
    auto fya = faces<const double>(fy, g, 1, NCONS);
    auto fza = faces<const double>(fz, g, 2, NCONS);
    auto fxsa = faces<const double>(fxs, g, 0, NSPECS);
    auto fysa = faces<const double>(fys, g, 1, NSPECS);
    auto fzsa = faces<const double>(fzs, g, 2, NSPECS);
    for_box(g, [&](int i, int j, int k) {
        for (int n = 0; n < NCONS; ++n) divop(i, j, k, n, dsdt, fxa, fya, fza, dxinv);
    });
    for_box(g, [&](int i, int j, int k) {
        for (int n = 0; n < NSPECS; ++n) divop(i, j, k, n, dsdts, fxsa, fysa, fzsa, dxinv);
    });
}

// Van Leer species flux of one face, Source/CHEM/FlowAdvanceBox.cpp:166-223.
static void eb_spec_flux(int i, int j, int k, int d, Array4<double> const& ql,
                         Array4<double> const& qr, Array4<double> const& rhol,
                         Array4<double> const& rhor, Array4<double> const& fs) {
    const int qn = d == 0 ? QU : (d == 1 ? QV : QW);
    amrex::GpuArray<Real, NSPECS> fp = {0}, fm = {0};
    Real ul, ur;
    ul = ql(i, j, k, qn);
    ur = qr(i, j, k, qn);
    Real cL = ql(i, j, k, QC);
    Real cR = qr(i, j, k, QC);
    Real ML, MR, UL, UR;
    ML = ul / cL;
    MR = ur / cR;
    UL = ul;
    UR = ur;
    if (ML >= 1.0) {
        for (int n = 0; n < NSPECS; ++n) fp[n] = rhol(i, j, k, n) * UL;
    } else if (amrex::Math::abs(ML) < 1.0) {
        Real Mp = 0.250 * (1.0 + ML) * (1.0 + ML);
        for (int n = 0; n < NSPECS; ++n) {
            Real tmp0 = rhol(i, j, k, n) * cL * Mp;
            fp[n] = tmp0;
        }
    }
    if (amrex::Math::abs(MR) < 1.0) {
        Real Mm = -0.250 * (MR - 1.0) * (MR - 1.0);
        for (int n = 0; n < NSPECS; ++n) {
            Real tmp0 = rhor(i, j, k, n) * cR * Mm;
            fm[n] = tmp0;
        }
    } else if (MR <= -1.0) {
        for (int n = 0; n < NSPECS; ++n) fm[n] = rhor(i, j, k, n) * UR;
    }
    for (int n = 0; n < NSPECS; ++n) fs(i, j, k, n) = fp[n] + fm[n];
}

// Cut-cell multispecies RHS, Source/CHEM/FlowAdvanceBox.cpp:105-499.
void ocfdr_rhs_chem_eb(const double* S, const double* spec, const uint32_t* flag_in,
                       const double* vfrac_in, const double* apx_in, const double* apy_in,
                       const double* apz_in, int nx, int ny, int nz, const double* dxinv_in,
                       int do_visc, double* dSdt, double* dSdt_spec, double* fx, double* fy,
                       double* fz, double* fxs, double* fys, double* fzs, double* fxd,
                       double* fyd, double* fzd) {
    Geo g{nx, ny, nz};
    Parm const& parm = the_parm();
    amrex::GpuArray<Real, 3> dxinv{{dxinv_in[0], dxinv_in[1], dxinv_in[2]}};
    amrex::GpuArray<Real, 3> weights{{0., 1., 0.5}};
    long long ng = g.gx() * g.gy() * g.gz();
    long long nn = (long long)(nx + 1) * (ny + 1) * (nz + 1);
    std::vector<double> qv(ng * NPRIM), qlv(nn * NPRIM, 1.0), qrv(nn * NPRIM, 1.0),
        rlv(nn * NSPECS, 1.0), rrv(nn * NSPECS, 1.0), divcv((long long)nx * ny * nz * NCONS, 0.0),
        muv(ng), lamv(ng), Dv(ng * NSPECS);
    auto s = grown<const double>(S, g, NCONS);
    auto spec_arr = grown<const double>(spec, g, NSPECS);
    auto q = grown<double>(qv.data(), g, NPRIM);
    auto ql = nodal<double>(qlv.data(), g, NPRIM);
    auto qr = nodal<double>(qrv.data(), g, NPRIM);
    auto rhol = nodal<double>(rlv.data(), g, NSPECS);
    auto rhor = nodal<double>(rrv.data(), g, NSPECS);
    auto mu = grown<double>(muv.data(), g, 1);
    auto lambda = grown<double>(lamv.data(), g, 1);
    auto D = grown<double>(Dv.data(), g, NSPECS);
    auto flag = grown<const amrex::EBCellFlag>(reinterpret_cast<const amrex::EBCellFlag*>(flag_in), g, 1);
    auto vfrac = grown<const double>(vfrac_in, g, 1);
    Array4<const double> apx = faces<const double>(apx_in, g, 0, 1);
    Array4<const double> apy = faces<const double>(apy_in, g, 1, 1);
    Array4<const double> apz = faces<const double>(apz_in, g, 2, 1);
    Array4<const double> none;
    auto dsdt_arr = interior<double>(dSdt, g, NCONS);
    auto dsdt_spec_arr = interior<double>(dSdt_spec, g, NSPECS);
    auto divc = interior<double>(divcv.data(), g, NCONS);
    double* fl[3] = {fx, fy, fz};
    double* fls[3] = {fxs, fys, fzs};
    double* fld[3] = {fxd, fyd, fzd};
    for (int d = 0; d < 3; ++d) {
        long long n = (long long)(nx + (d == 0)) * (ny + (d == 1)) * (nz + (d == 2));
        std::fill(fl[d], fl[d] + n * NCONS, 0.0);
        std::fill(fls[d], fls[d] + n * NSPECS, 0.0);
        if (do_visc) std::fill(fld[d], fld[d] + n * NSPECS, 0.0);
    }
    for_box(g, [&](int i, int j, int k) {
        for (int n = 0; n < NCONS; ++n) { dsdt_arr(i, j, k, n) = 0.0; divc(i, j, k, n) = 0.0; }
        for (int n = 0; n < NSPECS; ++n) dsdt_spec_arr(i, j, k, n) = 0.0;
    });
    for_grown(g, [&](int i, int j, int k) { c2prim_rgas(i, j, k, s, spec_arr, q, parm); });
    if (do_visc) transport(g, q, spec_arr, mu, lambda, D);
    for (int d = 0; d < 3; ++d) {
        auto f = faces<double>(fl[d], g, d, NCONS);
        auto fs = faces<double>(fls[d], g, d, NSPECS);
        for_faces(g, d, [&](int i, int j, int k) {
            for (int n = 0; n < NPRIM; ++n) {
                if (d == 0) eb_recon_x(i, j, k, n, vfrac, ql, qr, q, flag, parm);
                if (d == 1) eb_recon_y(i, j, k, n, vfrac, ql, qr, q, flag, parm);
                if (d == 2) eb_recon_z(i, j, k, n, vfrac, ql, qr, q, flag, parm);
            }
        });
        for_faces(g, d, [&](int i, int j, int k) {
            for (int n = 0; n < NSPECS; ++n) {
                if (d == 0) eb_recon_x(i, j, k, n, vfrac, rhol, rhor, spec_arr, flag, parm);
                if (d == 1) eb_recon_y(i, j, k, n, vfrac, rhol, rhor, spec_arr, flag, parm);
                if (d == 2) eb_recon_z(i, j, k, n, vfrac, rhol, rhor, spec_arr, flag, parm);
            }
        });
        for_faces(g, d, [&](int i, int j, int k) { eb_flux(i, j, k, ql, qr, f, d, parm); });
        for_faces(g, d, [&](int i, int j, int k) { eb_spec_flux(i, j, k, d, ql, qr, rhol, rhor, fs); });
        if (do_visc) {
            auto fd = faces<double>(fld[d], g, d, NSPECS);
            for_faces(g, d, [&](int i, int j, int k) {
                if (d == 0) diffusion_x(i, j, k, q, spec_arr, D, fs, fd, dxinv);
                if (d == 1) diffusion_y(i, j, k, q, spec_arr, D, fs, fd, dxinv);
                if (d == 2) diffusion_z(i, j, k, q, spec_arr, D, fs, fd, dxinv);
            });
            for_faces(g, d, [&](int i, int j, int k) {
                if (d == 0) compute_visc_x_multi_eb(i, j, k, q, spec_arr, lambda, mu, f, fd, flag, dxinv, weights, parm);
                if (d == 1) compute_visc_y_multi_eb(i, j, k, q, spec_arr, lambda, mu, f, fd, flag, dxinv, weights, parm);
                if (d == 2) compute_visc_z_multi_eb(i, j, k, q, spec_arr, lambda, mu, f, fd, flag, dxinv, weights, parm);
            });
        }
    }
    auto fxa = faces<double>(fx, g, 0, NCONS);
    auto fya = faces<double>(fy, g, 1, NCONS);
    auto fza = faces<double>(fz, g, 2, NCONS);
    auto fxsa = faces<double>(fxs, g, 0, NSPECS);
    auto fysa = faces<double>(fys, g, 1, NSPECS);
    auto fzsa = faces<double>(fzs, g, 2, NSPECS);
    // flow divergence into divc (dSdt stays zero: FlowAdvanceBox.cpp leaves the
    // divc -> dsdt copy commented out at :500-523)
    for_box(g, [&](int i, int j, int k) {
        if (do_visc)
            eb_compute_div_visc(i, j, k, q, divc, fxa, fya, fza, flag, vfrac, none, apx, apy, apz,
                                none, none, none, dxinv, parm);
        else
            eb_compute_div(i, j, k, q, divc, fxa, fya, fza, flag, vfrac, none, apx, apy, apz, none,
                           none, none, dxinv, parm);
    });
    for_box(g, [&](int i, int j, int k) {
        Real tmp = dxinv[0] / vfrac(i, j, k);
        if (flag(i, j, k).isCovered()) {
            for (int n = 0; n < NSPECS; ++n) dsdt_spec_arr(i, j, k, n) = Real(0.0);
        } else if (flag(i, j, k).isRegular()) {
            for (int n = 0; n < NSPECS; ++n)
                dsdt_spec_arr(i, j, k, n) = dxinv[0] * (fxsa(i + 1, j, k, n) - fxsa(i, j, k, n)) +
                                            dxinv[1] * (fysa(i, j + 1, k, n) - fysa(i, j, k, n)) +
                                            dxinv[2] * (fzsa(i, j, k + 1, n) - fzsa(i, j, k, n));
        } else {
            for (int n = 0; n < NSPECS; ++n)
                dsdt_spec_arr(i, j, k, n) =
                    tmp * (apx(i + 1, j, k) * fxsa(i + 1, j, k, n) - apx(i, j, k) * fxsa(i, j, k, n) +
                           apy(i, j + 1, k) * fysa(i, j + 1, k, n) - apy(i, j, k) * fysa(i, j, k, n) +
                           apz(i, j, k + 1) * fzsa(i, j, k + 1, n) - apz(i, j, k) * fzsa(i, j, k, n));
            if (do_visc) {
                amrex::GpuArray<Real, NSPECS> flux_wall;
                Real apnorm = std::sqrt((apx(i, j, k) - apx(i + 1, j, k)) * (apx(i, j, k) - apx(i + 1, j, k)) +
                                        (apy(i, j, k) - apy(i, j + 1, k)) * (apy(i, j, k) - apy(i, j + 1, k)) +
                                        (apz(i, j, k) - apz(i, j, k + 1)) * (apz(i, j, k) - apz(i, j, k + 1)));
                Real un = q(i, j, k, QU) * (apx(i, j, k) - apx(i + 1, j, k)) +
                          q(i, j, k, QV) * (apy(i, j, k) - apy(i, j + 1, k)) +
                          q(i, j, k, QW) * (apz(i, j, k) - apz(i, j, k + 1));
                Real lambda0 = amrex::Math::abs(un) + q(i, j, k, QC) * apnorm;
                for (int n = 0; n < NSPECS; ++n) {
                    Real fpw = 0.5 * (spec_arr(i, j, k, n) * un + lambda0 * spec_arr(i, j, k, n));
                    Real fmw = -0.5 * (spec_arr(i, j, k, n) * un + lambda0 * spec_arr(i, j, k, n));
                    flux_wall[n] = fpw + fmw;
                }
                for (int n = 0; n < NSPECS; ++n) dsdt_spec_arr(i, j, k, n) += flux_wall[n] * tmp;
            }
        }
        for (int n = 0; n < NSPECS; ++n) dsdt_spec_arr(i, j, k, n) *= -1.0;
    });
}
#endif

}  // extern "C"
