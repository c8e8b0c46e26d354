// Operation counts of OpenCFD-AMR's point functions (test and measurement
// infrastructure; make -C oracle flops builds this ideal-gas and, with -DCHEM
// and Source/Constants.cpp, multispecies).  The reference's kernel
// headers are compiled unmodified with amrex::Real = CountedReal
// (oracle/shim/flop_real.H); each function is called once at one point of a
// small state and the tally it leaves is printed as JSON.  The algorithmic
// FLOPs of one cell's right-hand side follow the chain of
// Source/Advance.cpp:245-329 per cell: c2prim once, the Steger-Warming split once
// per direction, WENO-Z for 5 components on one face per direction, the
// viscous flux on one face per direction, divop for 5 components.
#include <AMReX_FArrayBox.H>
#include <IndexDefines.H>
#include <Constants.H>
#include <Kernels.H>
#include <FluxSplit.H>
#include <Reconstruction.H>
#include <Diffusion.H>
#ifdef CHEM
#include <LiDryer.H>
#include <ChemViscous.H>
#endif

#include <cstdio>
#include <string>
#include <vector>

using amrex::Array4;
using amrex::Dim3;
using amrex::Real;

namespace {

constexpr int NG = 4, N = 2 * NG + 1;  // a 9^3 block around cell (0, 0, 0)

struct Block {
    std::vector<Real> data;
    Array4<Real> a;
    explicit Block(int nc) : data((size_t)nc * N * N * N) {
        a = Array4<Real>(data.data(), N, N * N, (long long)N * N * N, Dim3{-NG, -NG, -NG}, Dim3{NG + 1, NG + 1, NG + 1},
                         nc);
    }
};

FlopTally since(const FlopTally& t0) {
    const FlopTally& t = flop_tally();
    FlopTally d;
    d.add = t.add - t0.add;
    d.mul = t.mul - t0.mul;
    d.div = t.div - t0.div;
    d.sqrt = t.sqrt - t0.sqrt;
    d.cmp = t.cmp - t0.cmp;
    d.other = t.other - t0.other;
    return d;
}

void put(const char* name, const FlopTally& d, bool last = false) {
    std::printf("  \"%s\": {\"add\": %lld, \"mul\": %lld, \"div\": %lld, \"sqrt\": %lld, \"cmp\": %lld, "
                "\"other\": %lld}%s\n",
                name, d.add, d.mul, d.div, d.sqrt, d.cmp, d.other, last ? "" : ",");
}

}  // namespace

#ifdef CHEM
amrex::GpuArray<Real, 3> dxinv_of(const Parm&) { return amrex::GpuArray<Real, 3>{{Real(1e4), Real(1e4), Real(1e4)}}; }

// The multispecies build: one cell of H2/air (phi = 1) at 1500 K, 1 atm, with a
// few radicals.  Counts of the temperature inversion (its Newton iteration count
// depends on the state), the production rates with their Jacobian, the
// elimination, the whole implicit substep (the lambda of
// Source/CHEM/ChemAdvance.cpp:27-82, restated as the reference driver does) and
// the mixture-averaged transport of one cell.
int chem_main() {
    Parm parm;
    parm.Initialize();
    const Parm* lparm = &parm;
    Real X[NSPECS] = {0.28, 0.14, 0.02, 0.002, 0.001, 0.004, 0.0005, 0.0001, 0.0};
    Real xs = 0.0;
    for (int n = 0; n < NSPECS - 1; ++n) xs += X[n];
    X[NSPECS - 1] = 1.0 - xs;
    Real Y[NSPECS], rho, e, rhoi[NSPECS];
    CKXTY(X, Y, parm);
    CKRHOY(Real(101325.0), Real(1500.0), Y, rho, parm);
    for (int n = 0; n < NSPECS; ++n) rhoi[n] = rho * Y[n];
    CKUBMS(Real(1500.0), rhoi, e, parm);
    const Real ei = e, dt = 1.25e-9;
    std::printf("{\n");
    FlopTally t0 = flop_tally();
    Real T;
    {
        Real r[NSPECS];
        for (int n = 0; n < NSPECS; ++n) r[n] = rhoi[n];
        GET_T_GIVEN_EY(ei, r, T, parm);
    }
    put("get_t_given_ey", since(t0));
    Real cc[NSPECS], wdot[NSPECS], Arate[NSPECS][NSPECS];
    for (int n = 0; n < NSPECS; n++) cc[n] = rhoi[n] / lparm->mw[n] * 1e-6;
    t0 = flop_tally();
    vproductionRate(wdot, Arate, cc, T, parm);
    put("vproductionRate", since(t0));
    Real A1[NSPECS][NSPECS], b[NSPECS], x[NSPECS];
    for (int i = 0; i < NSPECS; ++i) {
        b[i] = wdot[i];
        for (int j = 0; j < NSPECS; ++j) A1[i][j] = (i == j ? 1.0 : 0.0) - Arate[i][j] * 1e-9;
    }
    t0 = flop_tally();
    gauss(x, A1, b);
    put("gauss", since(t0));
    // the whole substep of one cell (state at rest)
    t0 = flop_tally();
    {
        Real rhoi_0[NSPECS], wd[NSPECS], c2[NSPECS], Ar[NSPECS][NSPECS], B1[NSPECS][NSPECS], rhoi_1[NSPECS],
            drho[NSPECS], T2, dei = 0;
        const Real rr = amrex::max(rho, lparm->smallr);
        const Real rhoinv = Real(1.0) / rr;
        const Real ux = Real(0.0) * rhoinv, uy = Real(0.0) * rhoinv, uz = Real(0.0) * rhoinv;
        const Real kineng = Real(0.5) * (ux * ux + uy * uy + uz * uz);
        Real e2 = ei - rr * kineng;
        for (int n = 0; n < NSPECS; ++n) rhoi_0[n] = rhoi[n];
        GET_T_GIVEN_EY(e2, rhoi_0, T2, *lparm);
        for (int n = 0; n < NSPECS; n++) c2[n] = rhoi_0[n] / lparm->mw[n] * 1e-6;
        vproductionRate(wd, Ar, c2, T2, *lparm);
        for (int i = 0; i < NSPECS; ++i)
            for (int j = 0; j < NSPECS; ++j) {
                B1[i][j] = (i == j ? 1.0 : 0.0);
                B1[i][j] -= Ar[i][j] * lparm->mw[i] / lparm->mw[j] * dt;
            }
        for (int n = 0; n < NSPECS; ++n) rhoi_1[n] = wd[n] * lparm->mw[n] * 1e6 * dt;
        gauss(drho, B1, rhoi_1);
        Real out[NSPECS];
        for (int n = 0; n < NSPECS; ++n) {
            out[n] = rhoi_0[n] + drho[n];
            if (out[n] < 0) out[n] = Real(0.0);
        }
        for (int n = 0; n < NSPECS; ++n) dei += -lparm->HP[n] * lparm->Ru / lparm->mw[n] * drho[n];
        (void)out;
        (void)dei;
    }
    put("chemical_advance_cell", since(t0));
    Real mu, lam;
    t0 = flop_tally();
    mixtureProperties(T, X, mu, lam, parm);
    put("mixtureProperties", since(t0));
    std::vector<Real> Dv(NSPECS);
    Array4<Real> D(Dv.data(), 1, 1, 1, Dim3{0, 0, 0}, Dim3{1, 1, 1}, NSPECS);
    t0 = flop_tally();
    getMixDiffCoeffsMass(0, 0, 0, T, Real(101325.0), X, D, parm);
    put("getMixDiffCoeffsMass", since(t0));

    // The multispecies right-hand side of Source/CHEM/FlowAdvance.cpp:157-403 on a
    // 9^3 block of this mixture (slightly varied, moving): the per-cell pieces
    Block u(NCONS), sp(NSPECS), q(NPRIM), mub(1), lamb(1), Db(NSPECS), fp(NCONS), fm(NCONS), fps(NSPECS),
        fms(NSPECS), fx(NCONS), fxs(NSPECS), fxd(NSPECS), ds(NCONS), dss(NSPECS);
    for (int k = -NG; k <= NG; ++k)
        for (int j = -NG; j <= NG; ++j)
            for (int i = -NG; i <= NG; ++i) {
                const double f = 1.0 + 0.002 * (i + 2 * j + 3 * k);
                Real r = 0.0;
                for (int n = 0; n < NSPECS; ++n) {
                    sp.a(i, j, k, n) = rhoi[n] * f;
                    r += rhoi[n] * f;
                }
                u.a(i, j, k, URHO) = r;
                u.a(i, j, k, UMX) = r * 30.0;
                u.a(i, j, k, UMY) = r * -20.0;
                u.a(i, j, k, UMZ) = r * 10.0;
                u.a(i, j, k, UEDEN) = e * f + 0.5 * r * 1400.0;
            }
    Array4<Real const> uc = u.a, spc = sp.a;
    for (int k = -NG; k <= NG; ++k)
        for (int j = -NG; j <= NG; ++j)
            for (int i = -NG; i <= NG; ++i) {
                c2prim_rgas(i, j, k, uc, spc, q.a, parm);
                Real Yt[NSPECS], Xt[NSPECS];
                for (int n = 0; n < NSPECS; ++n) Yt[n] = sp.a(i, j, k, n) / q.a(i, j, k, QRHO);
                CKYTX(Yt, Xt, parm);
                mixtureProperties(q.a(i, j, k, QT), Xt, mub.a(i, j, k), lamb.a(i, j, k), parm);
                Array4<Real> Dij(&Db.a(i, j, k, 0), 1, 1, Db.a.nstride, Dim3{i, j, k}, Dim3{i + 1, j + 1, k + 1},
                                 NSPECS);
                getMixDiffCoeffsMass(i, j, k, q.a(i, j, k, QT), q.a(i, j, k, QPRES), Xt, Dij, parm);
            }
    Array4<Real const> qc = q.a, muc = mub.a, lamc = lamb.a, Dc = Db.a;
    t0 = flop_tally();
    c2prim_rgas(0, 0, 0, uc, spc, q.a, parm);
    put("c2prim_rgas", since(t0));
    t0 = flop_tally();
    {
        Real Yt[NSPECS], Xt[NSPECS], m1, l1;
        for (int n = 0; n < NSPECS; ++n) Yt[n] = sp.a(0, 0, 0, n) / q.a(0, 0, 0, QRHO);
        CKYTX(Yt, Xt, parm);
        mixtureProperties(q.a(0, 0, 0, QT), Xt, m1, l1, parm);
        std::vector<Real> D1(NSPECS);
        Array4<Real> Da(D1.data(), 1, 1, 1, Dim3{0, 0, 0}, Dim3{1, 1, 1}, NSPECS);
        getMixDiffCoeffsMass(0, 0, 0, q.a(0, 0, 0, QT), q.a(0, 0, 0, QPRES), Xt, Da, parm);
    }
    put("transport_cell", since(t0));
    for (int k = -NG; k <= NG; ++k)
        for (int j = -NG; j <= NG; ++j)
            for (int i = -NG; i <= NG; ++i) flux_split_x(i, j, k, fp.a, fm.a, qc, uc, parm);
    t0 = flop_tally();
    flux_split_x(0, 0, 0, fp.a, fm.a, qc, uc, parm);
    put("flux_split_x_chem", since(t0));
    // the species split lambda of Source/CHEM/FlowAdvance.cpp:214-242, restated
    auto spec_split = [&](int i, int j, int k) {
        Real un = q.a(i, j, k, QU), c = q.a(i, j, k, QC), gamma = q.a(i, j, k, QGAMA);
        Real E1 = un, E2 = un - c, E3 = un + c;
        Real E1P = (E1 + amrex::Math::abs(E1)) * Real(0.5);
        Real E2P = (E2 + amrex::Math::abs(E2)) * Real(0.5);
        Real E3P = (E3 + amrex::Math::abs(E3)) * Real(0.5);
        Real E1M = E1 - E1P, E2M = E2 - E2P, E3M = E3 - E3P;
        Real tmp1 = Real(1.0) / (Real(2.0) * gamma);
        Real tmp2 = Real(2.0) * (gamma - Real(1.0));
        Real tmp2_p = tmp2 * E1P + E2P + E3P;
        Real tmp2_m = tmp2 * E1M + E2M + E3M;
        for (int n = 0; n < NSPECS; ++n) {
            Real tmp0 = sp.a(i, j, k, n) * tmp1;
            fps.a(i, j, k, n) = tmp0 * tmp2_p;
            fms.a(i, j, k, n) = tmp0 * tmp2_m;
        }
    };
    for (int k = -NG; k <= NG; ++k)
        for (int j = -NG; j <= NG; ++j)
            for (int i = -NG; i <= NG; ++i) spec_split(i, j, k);
    t0 = flop_tally();
    spec_split(0, 0, 0);
    put("species_split_x", since(t0));
    Array4<Real const> fpc = fp.a, fmc = fm.a, fpsc = fps.a, fmsc = fms.a;
    t0 = flop_tally();
    reconstruction_x(0, 0, 0, 0, fpc, fmc, fx.a, parm);
    put("reconstruction_x_chem", since(t0));
    t0 = flop_tally();
    diffusion_x(0, 0, 0, qc, spc, Dc, fxs.a, fxd.a, dxinv_of(parm));
    put("diffusion_x", since(t0));
    Array4<Real const> fxdc = fxd.a;
    t0 = flop_tally();
    compute_visc_x_multi(0, 0, 0, qc, spc, lamc, muc, fx.a, fxdc, dxinv_of(parm), parm);
    put("compute_visc_x_multi", since(t0), true);
    (void)ds;
    (void)dss;
    std::printf("}\n");
    return 0;
}
#endif

int main() {
#ifdef CHEM
    return chem_main();
#endif
    Parm parm;
    parm.Rg = parm.Ru / parm.eos_m;
    parm.cp = parm.eos_gamma * parm.Rg / (parm.eos_gamma - 1.0);
    parm.cv = parm.cp / parm.eos_gamma;
    parm.kOverMu = parm.cp / parm.Pr;
    Block u(NCONS), q(NPRIM), fp(NCONS), fm(NCONS), fx(NCONS), fy(NCONS), fz(NCONS), dsdt(NCONS);
    // a smooth state: rho 1 +, velocity and pressure of order one
    for (int k = -NG; k <= NG; ++k)
        for (int j = -NG; j <= NG; ++j)
            for (int i = -NG; i <= NG; ++i) {
                const double r = 1.0 + 0.01 * (i + 2 * j + 3 * k + 20), vx = 0.3, vy = -0.2, vz = 0.1, p = 1.0;
                u.a(i, j, k, URHO) = r;
                u.a(i, j, k, UMX) = r * vx;
                u.a(i, j, k, UMY) = r * vy;
                u.a(i, j, k, UMZ) = r * vz;
                u.a(i, j, k, UEDEN) = p / 0.4 + 0.5 * r * (vx * vx + vy * vy + vz * vz);
            }
    Array4<Real const> uc = u.a;
    for (int k = -NG; k <= NG; ++k)
        for (int j = -NG; j <= NG; ++j)
            for (int i = -NG; i <= NG; ++i) c2prim(i, j, k, uc, q.a, parm);
    Array4<Real const> qc = q.a;
    amrex::GpuArray<Real, 3> dxinv{{Real(64.0), Real(64.0), Real(64.0)}};
    std::printf("{\n");
    FlopTally t0 = flop_tally();
    c2prim(0, 0, 0, uc, q.a, parm);
    put("c2prim", since(t0));
    const char* split_names[3] = {"flux_split_x", "flux_split_y", "flux_split_z"};
    const char* recon_names[3] = {"reconstruction_x", "reconstruction_y", "reconstruction_z"};
    const char* visc_names[3] = {"compute_visc_x", "compute_visc_y", "compute_visc_z"};
    for (int d = 0; d < 3; ++d) {
        for (int k = -NG; k <= NG; ++k)
            for (int j = -NG; j <= NG; ++j)
                for (int i = -NG; i <= NG; ++i) {
                    if (d == 0) flux_split_x(i, j, k, fp.a, fm.a, qc, uc, parm);
                    if (d == 1) flux_split_y(i, j, k, fp.a, fm.a, qc, uc, parm);
                    if (d == 2) flux_split_z(i, j, k, fp.a, fm.a, qc, uc, parm);
                }
        t0 = flop_tally();
        if (d == 0) flux_split_x(0, 0, 0, fp.a, fm.a, qc, uc, parm);
        if (d == 1) flux_split_y(0, 0, 0, fp.a, fm.a, qc, uc, parm);
        if (d == 2) flux_split_z(0, 0, 0, fp.a, fm.a, qc, uc, parm);
        put(split_names[d], since(t0));
        Array4<Real const> fpc = fp.a, fmc = fm.a;
        t0 = flop_tally();
        if (d == 0) reconstruction_x(0, 0, 0, 0, fpc, fmc, fx.a, parm);
        if (d == 1) reconstruction_y(0, 0, 0, 0, fpc, fmc, fy.a, parm);
        if (d == 2) reconstruction_z(0, 0, 0, 0, fpc, fmc, fz.a, parm);
        put(recon_names[d], since(t0));
        t0 = flop_tally();
        if (d == 0) compute_visc_x(0, 0, 0, qc, fx.a, dxinv, parm);
        if (d == 1) compute_visc_y(0, 0, 0, qc, fy.a, dxinv, parm);
        if (d == 2) compute_visc_z(0, 0, 0, qc, fz.a, dxinv, parm);
        put(visc_names[d], since(t0));
    }
    Array4<Real const> fxc = fx.a, fyc = fy.a, fzc = fz.a;
    t0 = flop_tally();
    divop(0, 0, 0, 0, dsdt.a, fxc, fyc, fzc, dxinv);
    put("divop", since(t0), true);
    std::printf("}\n");
    return 0;
}
