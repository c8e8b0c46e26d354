/* CPU oracle for the OpenCFD-AMR right-hand-side / update path.
 *
 * TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load this library, and only as the checker or the timed CPU
 * baseline, never as the thing that ships.
 *
 * A plain-C restatement of the reference's arithmetic, in the reference's
 * operation order, so that built with -ffp-contract=off it reproduces the
 * reference's own kernels (compiled from their sources by oracle/Makefile's `ref`
 * target) bit for bit; tests/test_oracle_vs_ref.py checks exactly that, and
 * tests/golden/ holds fixtures produced by the reference build.
 *
 * Array convention (same as oracle/ref/ref_driver.cpp): a box interior
 * [0,nx)x[0,ny)x[0,nz) with OCFDO_NG ghost cells; cell arrays over the grown
 * box, i fastest, component slowest; dSdt over the interior; face arrays of
 * direction d over the interior box made nodal in d.
 */
#ifndef OCFD_ORACLE_H
#define OCFD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OCFDO_NG 4
#define OCFDO_NSPEC 9

/* Mirror of the reference's Parm (Source/Constants.H:7-64) with the CHEM tables
 * held inline instead of behind device pointers. */
typedef struct {
    double eos_gamma, eos_m, Patm, cv, cp, Ru, Rg, kOverMu;
    double Pr, C_s, T_s, smallr, smallp, eps, twoThirds, oneSix;
    double mw[OCFDO_NSPEC];
    double nasa_lo[OCFDO_NSPEC][7];
    double nasa_hi[OCFDO_NSPEC][7];
    double HP[OCFDO_NSPEC];
    double A0[OCFDO_NSPEC];
    double visccoeff[OCFDO_NSPEC * 5];
    double conductcoeff[OCFDO_NSPEC * 5];
    double diffcoeff[45 * 5];
} ocfdo_parm;

void ocfdo_parm_default(ocfdo_parm* p);

/* ---- point-level thermochemistry (Source/CHEM/LiDryer.H, ChemViscous.H) ---- */
void ocfdo_ckxty(const ocfdo_parm* p, const double* x, double* y);
void ocfdo_ckytx(const ocfdo_parm* p, const double* y, double* x);
double ocfdo_ckrhoy(const ocfdo_parm* p, double P, double T, const double* y);
double ocfdo_ckubms(const ocfdo_parm* p, double T, const double* rhoi);
double ocfdo_ckcvbs(const ocfdo_parm* p, double T, const double* rhoi);
double ocfdo_ckpy(const ocfdo_parm* p, const double* rhoi, double T);
double ocfdo_get_t_given_ey(const ocfdo_parm* p, double e, const double* rhoi);
void ocfdo_production_rate(const ocfdo_parm* p, const double* c, double T, double* wdot,
                           double* arate /* 9x9 row-major */);
void ocfdo_gauss(const double* a /* 9x9 */, const double* b, double* x);
void ocfdo_mixture_properties(const ocfdo_parm* p, double T, const double* X, double* mu,
                              double* lambda);
void ocfdo_mix_diff_coeffs(const ocfdo_parm* p, double T, double P, const double* X, double* D);
void ocfdo_species_enthalpy(const ocfdo_parm* p, double T, double* h);

/* ---- box level ---- */
/* primitives over the grown box; chem != 0 uses the real-gas form with spec */
void ocfdo_c2prim(const ocfdo_parm* p, int chem, const double* S, const double* spec, int nx,
                  int ny, int nz, double* q);

/* do_visc: bit 0 the viscous flux (EBR::do_visc), bit 1 the gravity source
 * (EBR::do_gravity, Source/Advance.cpp:331-342) */
void ocfdo_rhs_regular(const ocfdo_parm* p, const double* S, int nx, int ny, int nz,
                       const double* dxinv, int do_visc, double* dSdt, double* fx, double* fy,
                       double* fz);

void ocfdo_rhs_eb(const ocfdo_parm* p, const double* S, const uint32_t* flag,
                  const double* vfrac, const double* apx, const double* apy, const double* apz,
                  int nx, int ny, int nz, const double* dxinv, int do_visc, int do_redistribute,
                  double* dSdt, double* fx, double* fy, double* fz);

void ocfdo_transport(const ocfdo_parm* p, const double* S, const double* spec, int nx, int ny,
                     int nz, double* mu, double* lambda, double* D);

void ocfdo_rhs_chem(const ocfdo_parm* p, const double* S, const double* spec, int nx, int ny,
                    int nz, const double* dxinv, int do_visc, double* dSdt, double* dSdt_spec,
                    double* fx, double* fy, double* fz, double* fxs, double* fys, double* fzs,
                    double* fxd, double* fyd, double* fzd);

void ocfdo_rhs_chem_eb(const ocfdo_parm* p, const double* S, const double* spec,
                       const uint32_t* flag, const double* vfrac, const double* apx,
                       const double* apy, const double* apz, int nx, int ny, int nz,
                       const double* dxinv, int do_visc, double* dSdt, double* dSdt_spec,
                       double* fx, double* fy, double* fz, double* fxs, double* fys,
                       double* fzs, double* fxd, double* fyd, double* fzd);

/* One semi-implicit chemistry substep, in place, over ncell cells whose
 * components are cstride apart (Source/CHEM/ChemAdvance.cpp:27-82). */
void ocfdo_chem_advance(const ocfdo_parm* p, double* S, double* spec, long long ncell,
                        long long cstride, double dt);

/* Species clip + rescale to the mixture density (Source/EBR.cpp:333-357). */
void ocfdo_spec_renorm(double* S, double* spec, long long ncell, long long cstride);

/* CFL time-step bound min over the interior of dx/(|u|+c)
 * (Source/Advance.cpp:10-59, without the cfl factor and the CHEM override). */
double ocfdo_estdt(const ocfdo_parm* p, const double* S, int nx, int ny, int nz,
                   const double* dx);

/* ---- single-level, single-box time stepping (test driver) ---- */
/* Physical boundary kinds per face, as in the reference's inputs lo_bc/hi_bc
 * (0 interior/periodic, 1 inflow, 2 outflow, 3 symmetry, 4 slip wall,
 * 5 no-slip wall), mapped to AMReX BC types by Source/Setup.cpp:17-92. */
typedef struct {
    int lo_bc[3], hi_bc[3];
    int dirichlet_case; /* 0 none, 1 double Mach reflection functor, 3 planar jet inflow */
    double prob_lo[3], dx[3];
    int dom_lo[3];      /* absolute index of the box's first interior cell */
    int dom_hi[3];      /* absolute index of the domain's last cell */
    double dmr_left[5], dmr_right[5];
    double jet[8];      /* rho_jet, u_jet, u_co, yc, w, delta, rho e, rho_co */
} ocfdo_bc;

void ocfdo_fill_ghosts(const ocfdo_bc* bc, double* S, int ncomp, int nx, int ny, int nz,
                       double time);

/* Advance nsteps SSP-RK3 steps of the ideal-gas regular-box scheme on a single
 * box that is the whole domain.  form 0 = Butcher-tableau form with stored stage
 * slopes (AMReX AmrLevel::RK(3)), form 1 = Shu-Osher convex form.  dt per step:
 * cfl*estdt, limited to 1.1x the previous step.  Returns the final time;
 * dts (nsteps entries, may be NULL) receives the steps taken. */
double ocfdo_advance_rk3(const ocfdo_parm* p, const ocfdo_bc* bc, double* S, int nx, int ny,
                         int nz, int do_visc, double cfl, int nsteps, int form, double* dts);
/* The same with ebr.time_integration = "RK2" (order 2, Heun) or "Euler"
 * (order 1), Source/Advance.cpp:115-138, in the reference's LinComb / Saxpy
 * operation order. */
double ocfdo_advance_rk12(const ocfdo_parm* p, const ocfdo_bc* bc, double* S, int nx, int ny,
                          int nz, int do_visc, double cfl, int nsteps, int order, double* dts);

/* One SSP-RK3 step of one box (regular scheme when flag is NULL, else the
 * cut-cell one) without ghost exchange between the stages, in place: the unit
 * the CPU baseline times on a sample of a hierarchy's boxes. */
void ocfdo_box_rk3_step(const ocfdo_parm* p, double* S, const uint32_t* flag, const double* vfrac,
                        const double* apx, const double* apy, const double* apz, int nx, int ny, int nz,
                        const double* dxinv, int do_redistribute, double dt);

#ifdef __cplusplus
}
#endif
#endif
