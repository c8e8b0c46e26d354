/* ocfd.h - C ABI of the GB300 (sm_103a) right-hand-side and update path for
 * OpenCFD-AMR.
 *
 * Every entry point is stream-ordered, takes plain pointers and sizes, returns an
 * ocfd_status and never traps on the device.  Device-side failures (a non-finite
 * value found by a checking kernel, a bounded wait that ran out) set a
 * per-context error word read by ocfd_context_check().
 *
 * Data layout mirrors AMReX so a caller can pass its own objects:
 *   ocfd_array4  has the member order and types of amrex::Array4<double>
 *                (p, jstride, kstride, nstride, begin, end, ncomp; begin/end are
 *                Dim3 = three ints, end exclusive), element (i,j,k,n) at
 *                p[(i-begin[0]) + (j-begin[1])*jstride + (k-begin[2])*kstride + n*nstride];
 *   ocfd_box     holds amrex::Box smallEnd/bigEnd (inclusive cell indices);
 *   ocfd_parm    has the member order of the reference's Parm
 *                (Source/Constants.H:7-64, CHEM build); a non-CHEM Parm is
 *                layout-identical to its first 16 doubles.
 * State arrays carry OCFD_NUM_GROW ghost cells (Source/EBR.H:207); face
 * arrays of direction d cover amrex::surroundingNodes(bx, d).
 */
#ifndef OCFD_OCFD_H
#define OCFD_OCFD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OCFD_NUM_GROW 4
#define OCFD_NCONS 5
#define OCFD_NSPEC 9

typedef enum ocfd_status {
    OCFD_OK = 0,
    OCFD_BAD_ARG = 1,        /* argument checks failed; nothing was launched */
    OCFD_LAUNCH_FAIL = 2,    /* a CUDA launch or runtime call failed */
    OCFD_TIMEOUT = 3,        /* a bounded device wait ran out */
    OCFD_NONFINITE = 4,      /* a checking kernel found NaN/Inf */
    OCFD_GUARD_FALLBACK = 5, /* a surrogate guard rejected cells (they were redone in FP64) */
    OCFD_NO_DEVICE = 6,      /* no CUDA device, or the device is not sm_103 */
    OCFD_OUT_OF_MEMORY = 7,
    OCFD_UNSUPPORTED = 8     /* valid request this build does not serve */
} ocfd_status;

/* amrex::Array4<double> */
typedef struct ocfd_array4 {
    double* p;
    int64_t jstride, kstride, nstride;
    int32_t begin[3];
    int32_t end[3];
    int32_t ncomp;
} ocfd_array4;

/* amrex::Array4<amrex::EBCellFlag const>: 32-bit flag words.  Bits 0-1 cell
 * type (0 regular, 1 single-valued cut, 3 covered); bit 4+(i+1)+3(j+1)+9(k+1)
 * set when the neighbour at offset (i,j,k) is connected. */
typedef struct ocfd_flag4 {
    const uint32_t* p;
    int64_t jstride, kstride, nstride;
    int32_t begin[3];
    int32_t end[3];
    int32_t ncomp;
} ocfd_flag4;

/* amrex::Box: inclusive cell-centred bounds */
typedef struct ocfd_box {
    int32_t lo[3];
    int32_t hi[3];
} ocfd_box;

/* Parm, Source/Constants.H:7-64 (CHEM member set).  Table pointers may be NULL
 * (the built-in Li-Dryer tables of Source/Constants.cpp:15-150 are used) or
 * point to host or device memory holding the reference's table layout.  The
 * floors smallr and smallp must be >= 0 (ocfd_context_create: OCFD_BAD_ARG). */
typedef struct ocfd_parm {
    double eos_gamma, eos_m, Patm;
    double cv, cp, Ru, Rg, kOverMu;
    double Pr, C_s, T_s;
    double smallr, smallp, eps;
    double twoThirds, oneSix;
    const double* mw;
    const double *H2_lo, *H2_hi, *O2_lo, *O2_hi, *H2O_lo, *H2O_hi, *H_lo, *H_hi, *O_lo, *O_hi;
    const double *OH_lo, *OH_hi, *HO2_lo, *HO2_hi, *H2O2_lo, *H2O2_hi, *N2_lo, *N2_hi;
    const double* HP;
    const double* A0;
    const double* visccoeff;
    const double* conductcoeff;
    const double* diffcoeff;
} ocfd_parm;

/* Flags of the RHS entry points */
#define OCFD_VISC 1u           /* EBR::do_visc (Source/EBR.cpp:25) */
#define OCFD_REDISTRIBUTE 2u   /* EBR::do_redistribute (Source/EBR.cpp:27), cut boxes only */
#define OCFD_FLUX_FP32 4u      /* mixed precision: split + WENO-Z in FP32, FP64 divergence */
#define OCFD_GRAVITY 16u       /* EBR::do_gravity (Source/EBR.cpp:26): dSdt(UMZ) += g rho, dSdt(UEDEN) += g rho w
                                  with g = -9.8 in regular boxes (Source/Advance.cpp:331-342) */
#define OCFD_PER_BOX 8u        /* level / hierarchy steps: the reference's execution model - every
                                  box's RHS stage as its own launches, issued from the host each
                                  step (no graph); for comparison with the batched graph form */

typedef struct ocfd_context ocfd_context;

/* ---------------------------------------------------------------- setup */
/* Reference defaults (Source/Constants.H:9-30) followed by Parm::Initialize
 * (Source/Constants.cpp:7-12); table pointers set to the library's host copies
 * of the Li-Dryer data.  Host only; needs no device. */
ocfd_status ocfd_parm_default(ocfd_parm* parm);

/* Binds `device`, uploads the mechanism tables and allocates the context's
 * scratch pool and error word.  One context per host thread and stream. */
ocfd_status ocfd_context_create(const ocfd_parm* parm, int device, ocfd_context** ctx);
ocfd_status ocfd_context_destroy(ocfd_context* ctx);

/* Synchronises `stream`, returns the device error word (0 = none) and clears it.
 * Returns OCFD_NONFINITE / OCFD_TIMEOUT when the word says so. */
ocfd_status ocfd_context_check(ocfd_context* ctx, void* stream, uint32_t* device_error);

const char* ocfd_status_string(ocfd_status s);
/* Message of the last failing call on this host thread ("" if none). */
const char* ocfd_last_error(void);
/* Library version, and the compute capability it was built for (e.g. 1030). */
int ocfd_version(void);
int ocfd_built_arch(void);

/* ------------------------------------------------------- box right-hand sides */
/* Regular (uncut) box, ideal gas: c2prim -> Steger-Warming split -> WENO-Z face
 * flux (+ viscous flux with OCFD_VISC) -> divergence, for all three directions,
 * in one fused launch.  Replaces the kernel chain of EBR::compute_dSdt,
 * Source/Advance.cpp:231-329 (point kernels Source/kernel/Kernels.H:13-40,84-97,
 * FluxSplit.H:11-193, Reconstruction.H:70-279, Diffusion.H:7-131).
 *   S     state, ncomp >= 5, covering grow(bx, 4)
 *   dSdt  output over bx, ncomp >= 5
 *   flux  NULL or three face arrays (x, y, z) over surroundingNodes(bx, d) that
 *         receive the face fluxes the reflux registers consume (Advance.cpp:219-222)
 *   dxinv inverse cell sizes (geom.InvCellSizeArray()) */
ocfd_status ocfd_rhs_regular_box_f64(ocfd_context* ctx, const ocfd_array4* S,
                                     const ocfd_array4* dSdt, const ocfd_array4* flux,
                                     ocfd_box bx, const double dxinv[3], unsigned flags,
                                     void* stream);

/* Cut-cell box (grow(bx,4) contains a cut cell), ideal gas: MUSCL-minmod
 * reconstruction of the primitives where the neighbours are connected, Van Leer
 * flux (+ EB-aware viscous flux with OCFD_VISC), cut-cell divergence with the
 * wall flux, negated; OCFD_REDISTRIBUTE applies the reference's local rescale.
 * Replaces EBR::eb_compute_dSdt_box, Source/EB/AdvanceBox.cpp:16-228 (point
 * kernels Source/EB/EBkernels.H:9-377, EBdiffusion.H:8-203).
 *   S       state covering grow(bx, 2), ncomp >= 5
 *   flag    EBCellFlag words covering grow(bx, 1)
 *   vfrac   volume fractions covering bx
 *   apx/apy/apz  area fractions over surroundingNodes(bx, d)
 *   fc, bcent    face / boundary centroids: accepted for interface fidelity and
 *                not read (the reference passes them and does not read them)
 * Scratch comes from the context pool. */
ocfd_status ocfd_rhs_eb_box_f64(ocfd_context* ctx, const ocfd_array4* S, const ocfd_array4* dSdt,
                                const ocfd_array4* flux, const ocfd_flag4* flag,
                                const ocfd_array4* vfrac, const ocfd_array4* apx,
                                const ocfd_array4* apy, const ocfd_array4* apz,
                                const ocfd_array4* const* fc, const ocfd_array4* bcent,
                                ocfd_box bx, const double dxinv[3], unsigned flags, void* stream);

/* Same computation as ocfd_rhs_eb_box_f64, for callers that cannot let a
 * library allocate device memory (applications that own all device memory
 * through their own pool, or code where a cudaMalloc/cudaFree, which can
 * synchronise the device, must not happen).  It has no counterpart in the
 * reference.  Its scratch is a fixed 16 MiB array compiled into the library
 * (2^21 doubles), held by every GPU that loads the library until exit; a box
 * needing more (7 (nx+4)(ny+4)(nz+4) doubles, plus 5 per face of the three face
 * boxes when flux is NULL) is rejected with OCFD_BAD_ARG.  It allocates nothing.
 * ocfd_context_create looks up the array's device address for its device and
 * loads the device code of this call, so the array is resident from context
 * creation on and no call loads anything; the context's device must be current
 * at each call.  All calls share the array, which keeps what the last call left:
 * calls that overlap on the GPU race and must be serialised by the caller. */
ocfd_status ocfd_rhs_eb_box_f64_static_scratch(
    ocfd_context* ctx, const ocfd_array4* S, const ocfd_array4* dSdt, const ocfd_array4* flux,
    const ocfd_flag4* flag, const ocfd_array4* vfrac, const ocfd_array4* apx,
    const ocfd_array4* apy, const ocfd_array4* apz, const ocfd_array4* const* fc,
    const ocfd_array4* bcent, ocfd_box bx, const double dxinv[3], unsigned flags, void* stream);

/* Regular box, multispecies (9-species Li-Dryer gas): real-gas primitives (T by
 * Newton on NASA-7, p from the species, gamma = 1 + p/e), Steger-Warming split of
 * the flow with the local gamma and of the species densities, WENO-Z of all
 * 5 + 9 components, and with OCFD_VISC mixture-averaged transport (Wilke
 * viscosity, averaged conductivity, mixture-averaged Fick diffusion) with the
 * species-enthalpy flux; divergence of both.  Replaces the regular-box branch of
 * EBR::compute_dSdt_multi, Source/CHEM/FlowAdvance.cpp:157-403.
 *   S, spec        covering grow(bx, 4) (5 and 9 components)
 *   dSdt, dSdt_spec over bx
 *   flux, flux_spec NULL or three face arrays over surroundingNodes(bx, d) */
ocfd_status ocfd_rhs_chem_box_f64(ocfd_context* ctx, const ocfd_array4* S, const ocfd_array4* spec,
                                  const ocfd_array4* dSdt, const ocfd_array4* dSdt_spec,
                                  const ocfd_array4* flux, const ocfd_array4* flux_spec,
                                  ocfd_box bx, const double dxinv[3], unsigned flags,
                                  void* stream);

/* Cut-cell box, multispecies: MUSCL-minmod of the 8 primitives and 9 partial
 * densities, Van Leer flow flux (gamma averaged over the face) and species flux,
 * Fick diffusion + EB-aware multispecies viscous flux with OCFD_VISC, cut-cell
 * species divergence, negated.  As in the reference, the flow dSdt of a cut
 * multispecies box is left zero (its divc -> dSdt copy is commented out,
 * Source/CHEM/FlowAdvanceBox.cpp:500-523); the flow face fluxes are still
 * produced for reflux.  Replaces EBR::ebchem_compute_dSdt_box,
 * Source/CHEM/FlowAdvanceBox.cpp:16-525.
 *   S, spec covering grow(bx, 2); flag covering grow(bx, 1); vfrac over bx;
 *   apx/apy/apz over surroundingNodes(bx, d); fc/bcent not read */
ocfd_status ocfd_rhs_chem_eb_box_f64(ocfd_context* ctx, const ocfd_array4* S,
                                     const ocfd_array4* spec, const ocfd_array4* dSdt,
                                     const ocfd_array4* dSdt_spec, const ocfd_array4* flux,
                                     const ocfd_array4* flux_spec, const ocfd_flag4* flag,
                                     const ocfd_array4* vfrac, const ocfd_array4* apx,
                                     const ocfd_array4* apy, const ocfd_array4* apz,
                                     const ocfd_array4* const* fc, const ocfd_array4* bcent,
                                     ocfd_box bx, const double dxinv[3], unsigned flags,
                                     void* stream);

/* ------------------------------------------------------------ chemistry */
/* One linearised backward-Euler chemistry substep of length dt on every cell
 * of bx, in place: T from e by bounded Newton on NASA-7 (LiDryer.H:833-888),
 * Li-Dryer rates and analytic Jacobian (LiDryer.H:156-529), partial-pivot
 * solve of (I - dt W J W^-1) drho = dt W wdot (LiDryer.H:890-942), species
 * clipped at 0 and the formation-enthalpy change moved into rho E.  Replaces the
 * kernel of EBR::chemical_advance, Source/CHEM/ChemAdvance.cpp:7-85 (the caller
 * skips covered boxes as the reference does).
 *   S (>= 5 comps) and spec (9 partial densities) covering bx, updated in place */
ocfd_status ocfd_chem_advance_box_f64(ocfd_context* ctx, const ocfd_array4* S,
                                      const ocfd_array4* spec, ocfd_box bx, double dt,
                                      void* stream);

/* Clip negative partial densities and rescale them to sum to rho, in place
 * (EBR::post_timestep, Source/EBR.cpp:333-357). */
ocfd_status ocfd_spec_renorm_box_f64(ocfd_context* ctx, const ocfd_array4* S,
                                     const ocfd_array4* spec, ocfd_box bx, void* stream);

/* ------------------------------------------------------------------ level */
/* One AMR level advanced on the device: the build's own host driver in place of
 * AMReX's AmrLevel machinery (absent).  It owns the level's state FABs (each
 * box grown by OCFD_NUM_GROW), fills ghost cells on the device (same-level
 * exchange with periodic images, then the physical boundary types of
 * Source/Setup.cpp:17-92 and the case boundary functor, direction by
 * direction), and advances SSP-RK3 steps whose stages are fused RHS + update
 * launches over every box of the level (Source/Advance.cpp:81-150), with the
 * CFL step (Source/Advance.cpp:10-79, limited to 1.1x the previous step as
 * Source/EBR.cpp:268-275) reduced on the device.  A whole step is one CUDA
 * graph launch. */
typedef struct ocfd_level ocfd_level;

#define OCFD_BC_INTERIOR 0
#define OCFD_BC_INFLOW 1
#define OCFD_BC_OUTFLOW 2
#define OCFD_BC_SYMMETRY 3
#define OCFD_BC_SLIPWALL 4
#define OCFD_BC_NOSLIPWALL 5

#define OCFD_CASE_NONE 0
#define OCFD_CASE_DMR 1    /* Exec/1_DMR/prob_bcfill.cpp:9-59; params = left state (5), right state (5) */
#define OCFD_CASE_INFLOW 2 /* constant inflow state on ext_dir faces; params = state (5) */
/* planar jet entering through an ext_dir x-lo face: with s(y) = (1 + tanh((w -
 * |y - yc|) / delta)) / 2, u = u_co + (u_jet - u_co) s, rho = rho_co + (rho_jet -
 * rho_co) s, v = w = 0, uniform pressure; params = rho_jet, u_jet, u_co, yc, w,
 * delta, rho e (internal energy per volume), rho_co */
#define OCFD_CASE_JET 3

typedef struct ocfd_level_desc {
    int32_t nbox;
    const ocfd_box* boxes;   /* valid boxes: disjoint, inside the domain (else OCFD_BAD_ARG) */
    ocfd_box domain;         /* problem domain in cell indices of this level */
    int32_t lo_bc[3];        /* ebr.lo_bc codes, OCFD_BC_* (0 = periodic) */
    int32_t hi_bc[3];
    double dx[3];
    double prob_lo[3];
    int32_t bc_case;         /* OCFD_CASE_* */
    double case_params[16];
    int32_t tile;            /* regular-RHS tile shape index, -1 = automatic */
} ocfd_level_desc;

ocfd_status ocfd_level_create(ocfd_context* ctx, const ocfd_level_desc* desc, ocfd_level** level);
ocfd_status ocfd_level_destroy(ocfd_level* level);
/* Array4 (device) of box `ibox` of the level's current state. */
ocfd_status ocfd_level_state(ocfd_level* level, int ibox, ocfd_array4* out);
/* Copy the grown state FAB of every box from / to `buf` (host or device memory,
 * boxes back to back in box order, each (ncomp, nz+8, ny+8, nx+8), i fastest). */
ocfd_status ocfd_level_copy_in(ocfd_level* level, const double* buf, void* stream);
ocfd_status ocfd_level_copy_out(ocfd_level* level, double* buf, void* stream);
/* The same for the valid cells only (the level's state without ghost cells, as
 * an AMReX MultiFab copy of valid regions): `buf` holds box after box in box
 * order, each (ncomp, nz, ny, nx), i fastest - ocfd_level_valid_elems doubles.
 * Host buffers go through a device staging list (one copy each way) and a
 * gather / scatter kernel; device buffers are scattered / gathered directly.
 * Ghost cells keep their values: every step fills them before it reads them.
 * copy_valid_in resets the level's time to 0 as ocfd_level_copy_in does. */
ocfd_status ocfd_level_copy_valid_in(ocfd_level* level, const double* buf, void* stream);
ocfd_status ocfd_level_copy_valid_out(ocfd_level* level, double* buf, void* stream);
int64_t ocfd_level_valid_elems(const ocfd_level* level);
size_t ocfd_level_state_elems(const ocfd_level* level);
ocfd_status ocfd_level_fill_ghosts(ocfd_level* level, double time, void* stream);
/* Advance `nsteps` SSP-RK3 steps with CFL number `cfl` (flags: OCFD_VISC,
 * OCFD_FLUX_FP32).  Time and dt stay on the device; read them with
 * ocfd_level_time(). */
ocfd_status ocfd_level_advance(ocfd_level* level, int nsteps, double cfl, unsigned flags,
                               void* stream);
ocfd_status ocfd_level_time(ocfd_level* level, double* time, double* last_dt, void* stream);
/* Set the level time and forget the previous dt (the next step is not limited). */
ocfd_status ocfd_level_set_time(ocfd_level* level, double time, void* stream);

/* Steps that would pass `stop_time` are shortened to end on it, and later steps
 * have dt = 0 (stop-time limit of EBR::computeNewDt, Source/EBR.cpp:277-286).
 * Default: no stop time. */
ocfd_status ocfd_level_set_stop_time(ocfd_level* level, double stop_time, void* stream);

/* Cells of the level (valid cells of all boxes). */
int64_t ocfd_level_cells(const ocfd_level* level);
/* Kernels one ocfd_level_advance step launches with `flags`. */
int ocfd_level_launches_per_step(const ocfd_level* level, unsigned flags);
/* Average duration in ms of the level's fused RK-stage kernel (SSP-RK3's
 * stage 2 whatever the level's time integration: reads two states, writes one)
 * over `reps` back-to-back launches, timed with CUDA events on `stream`.
 * Overwrites the level's stage scratch buffer only. */
/* Device time of one part of a stage launch, averaged over `reps` (CUDA events
 * on `stream`; the launches write scratch only): part 0 the whole stage (as
 * ocfd_level_profile_stage), part 1 the regular boxes' tile kernel alone.
 * *cells (nullable) receives the cells that part covers.  No counterpart in the
 * reference (measurement). */
ocfd_status ocfd_level_profile_part(ocfd_level* level, unsigned flags, int part, int reps, double* ms,
                                    int64_t* cells, void* stream);
ocfd_status ocfd_level_profile_stage(ocfd_level* level, unsigned flags, int reps, double* ms,
                                     void* stream);

/* Autotuner of the batched stage kernel: times every tile shape that fits x
 * every tile schedule (0: one CTA per tile; 1: persistent CTAs striding over
 * the tiles; 2: persistent CTAs taking tiles from a work queue) over the
 * level's own boxes - `reps` launches each after a warm-up, CUDA events on
 * `stream` - and keeps the fastest.  Results do not depend on the choice
 * (bit-identical).  Overwrites the level's stage scratch buffer; synchronous.
 * tile / sched (may be NULL) receive the choice. */
ocfd_status ocfd_level_autotune(ocfd_level* level, unsigned flags, int reps, int32_t* tile, int32_t* sched,
                                void* stream);
/* Set the tile shape (index, -1 keeps it) and schedule (0-2) explicitly.  Tile
 * indices 0-5 are the pencil shapes (8,8,8), (8,8,4), (16,8,4), (16,16,2),
 * (32,8,2), (16,8,2); 6-8 the TMA-staged variants of the first three, which
 * stage in the inviscid FP32-flux form and run the pencil kernel otherwise.
 * A shape whose shared memory does not fit the form a step asks for makes
 * that step fail with OCFD_BAD_ARG. */
ocfd_status ocfd_level_set_schedule(ocfd_level* level, int32_t tile, int32_t sched);
/* Time integration of a standalone ideal-gas level, ebr.time_integration
 * (Source/EBR.cpp:36, Source/Advance.cpp:115-149): 3 = SSP-RK3 (the default
 * here; AmrLevel::RK(3, ...)), 2 = "RK2", Heun (U* = U^n + dt L(U^n), ghosts at
 * t; U^{n+1} = U^n/2 + (U* + dt L(U*))/2, ghosts at t + dt; the reference's
 * default), 1 = "Euler" (U^{n+1} = U^n + dt L(U^n), then a state copy).  The CFL
 * bound of the new state is fused into the last stage.  Synchronous; levels of a
 * hierarchy follow ocfd_amr_set_time_integration (OCFD_BAD_ARG here). */
ocfd_status ocfd_level_set_time_integration(ocfd_level* level, int32_t order);

/* ------------------------------------------- embedded boundary on a level
 * The box loop of EBR::compute_dSdt (Source/Advance.cpp:201-342) over a level
 * that an embedded body cuts: a box whose cells are all covered gets a zero
 * right-hand side (:213-214), a box whose grow(bx, 4) holds no cut or covered
 * cell takes the fused regular path (:231), every other box the cut-cell scheme
 * of eb_compute_dSdt_box (Source/EB/AdvanceBox.cpp:16-228: MUSCL-minmod, Van
 * Leer, cut-cell divergence with the wall flux).  The cut and covered boxes of
 * a level are batched: three launches per RK stage (primitives, faces of all
 * three directions, divergence fused with the RK stage update and the CFL
 * bound) beside the regular boxes' launch, inside the same step graph.  The
 * cut-cell scheme runs in FP64 in the plain form; with OCFD_FLUX_FP32 (inviscid)
 * its primitives, face states, Van Leer flux and divergence are FP32 and the RK
 * stage update stays FP64.
 *
 * AMReX's EB2 (Source/Geometry.cpp:9-29) is absent: the geometry is built on
 * the device from an implicit function by sub-sampling - flags with the
 * 27-neighbour connectivity (fluid neighbour, open shared face), volume
 * fractions, area fractions - for bodies extruded along z, stored per box as
 * z-invariant arrays (kstride 0) over grow(bx, 5) in x and y. */
#define OCFD_EB_NONE 0
#define OCFD_EB_CYLINDER_Z 1 /* fluid where (x-cx)^2 + (y-cy)^2 > r^2 */

typedef struct ocfd_eb_desc {
    int32_t kind;            /* OCFD_EB_* */
    int32_t nsub;            /* sub-samples per cell edge (0: 16) */
    double center[2];        /* axis position (x, y) */
    double radius;
    int32_t redistribute;    /* ebr.do_redistribute (Source/EBR.cpp:27; default 0) */
} ocfd_eb_desc;

#define OCFD_BOX_REGULAR 0
#define OCFD_BOX_CUT 1
#define OCFD_BOX_COVERED 2

/* Build the geometry of every box of the level, classify the boxes and rebuild
 * the stage tables (kind OCFD_EB_NONE removes the body).  Synchronous. */
ocfd_status ocfd_level_set_eb(ocfd_level* level, const ocfd_eb_desc* eb);
/* Class (OCFD_BOX_*) of every box, in box order. */
ocfd_status ocfd_level_box_classes(const ocfd_level* level, int32_t* classes);
/* Device views of the geometry of box `ibox` (a cut box; z-invariant, kstride
 * 0): flags and volume fractions over grow(bx, 5) in x, y; area fractions
 * ap[0..2] on the faces of grow(bx, 5) (ap[2], the z faces of an extruded body,
 * is the volume fraction). */
ocfd_status ocfd_level_eb_geometry(const ocfd_level* level, int ibox, ocfd_flag4* flag,
                                   ocfd_array4* vfrac, ocfd_array4* ap);
/* The same geometry copied to host arrays, rows of x: flag and vfrac (gy, gx),
 * apx (gy, gx + 1), apy (gy + 1, gx), gx = nx + 10, gy = ny + 10. */
ocfd_status ocfd_level_eb_geometry_copy(const ocfd_level* level, int ibox, uint32_t* flag, double* vfrac,
                                        double* apx, double* apy);

/* ------------------------------------------------------- reacting level (GPU)
 * A level of the multispecies flow with operator-split chemistry, one CUDA graph
 * per step: n chemistry substeps of dt/(2n), the flow step (RK2 as
 * Source/CHEM/FlowAdvance.cpp:95-122, or SSP-RK3) with the multispecies RHS of
 * every box, n substeps of dt/(2n), species renormalisation (EBR::advance CHEM
 * branch, Source/Advance.cpp:152-177; EBR::post_timestep, Source/EBR.cpp:333-357).
 * The level's FABs hold 14 components: the 5 conserved then the 9 partial
 * densities.  dt is fixed (the reference's CHEM time step, Source/Advance.cpp:54-57,
 * times its CFL number).                                                        */
typedef struct ocfd_react ocfd_react;

typedef struct ocfd_react_desc {
    ocfd_level_desc level;
    int32_t rk_order;        /* 2 (the reference) or 3 */
    int32_t chem_substeps;   /* per half step; 4 on level 0 (Source/Advance.cpp:159-161) */
    double dt;
    uint32_t flags;          /* OCFD_VISC: mixture-averaged viscous and species transport;
                                OCFD_FLUX_FP32: the mixed form - Steger-Warming split and WENO-Z of
                                the flow and species face fluxes in FP32 (primitives with the Newton
                                temperature, transport, viscous / diffusive fluxes, RK and chemistry
                                stay FP64) */
    int32_t binned_chem;     /* 1: chemistry as one launch over all cells ordered by a temperature key */
} ocfd_react_desc;

ocfd_status ocfd_react_create(ocfd_context* ctx, const ocfd_react_desc* desc, ocfd_react** react);
ocfd_status ocfd_react_destroy(ocfd_react* react);
/* The 14-component level: ocfd_level_copy_in / copy_out / time / cells. */
ocfd_level* ocfd_react_level(ocfd_react* react);
ocfd_status ocfd_react_advance(ocfd_react* react, int nsteps, void* stream);
/* Kernels of one step (the captured graph). */
int ocfd_react_launches_per_step(const ocfd_react* react);
/* Cut the reacting level with an embedded body (ocfd_eb_desc, see
 * ocfd_level_set_eb): the box loop of EBR::compute_dSdt_multi
 * (Source/CHEM/FlowAdvance.cpp:92-496) - covered boxes get a zero right-hand
 * side, regular boxes the multispecies chain, cut boxes the cut-cell chain of
 * ebchem_compute_dSdt_box (Source/CHEM/FlowAdvanceBox.cpp:16-525, FP64 in every
 * form) on the level's geometry - and the chemistry skips covered boxes
 * (Source/CHEM/ChemAdvance.cpp:20).  kind OCFD_EB_NONE removes the body.
 * Synchronous.  ocfd_react_box_classes: OCFD_BOX_* per box. */
ocfd_status ocfd_react_set_eb(ocfd_react* react, const ocfd_eb_desc* eb);
ocfd_status ocfd_react_box_classes(const ocfd_react* react, int32_t* cls);
/* Mean device time of one chemistry substep over the level (the configured
 * form), `reps` substeps of dt/(2 n) applied to the current state. */
ocfd_status ocfd_react_profile_chem(ocfd_react* react, int reps, double* ms, void* stream);
/* Conserved state of resting mixtures from temperature, pressure and mole
 * fractions (CKXTY, CKRHOY, CKUBMS as Exec/7_JET/prob.H:46-60 uses them), n
 * cells, device arrays: T[n], p[n], X[9][n] -> U[5][n] (rho, 0, 0, 0, rho e),
 * rhoY[9][n]. */
ocfd_status ocfd_chem_state_tpx(ocfd_context* ctx, int64_t n, const double* T, const double* p, const double* X,
                                double* U, double* rhoY, void* stream);

/* ---------------------------------------------------- AMR hierarchy (GPU)
 * The per-level path of EBR::advance / EBR::post_timestep run over a whole
 * refined hierarchy with subcycling in time (AMReX Amr::timeStep, ratio 2):
 *   - coarse-fine ghost cells of a finer level are interpolated from the coarser
 *     level with MC-limited conservative linear slopes, in time from the coarse
 *     SSP-RK3 stage states (the role of FillPatch / FillPatcher::fillRK under
 *     AmrLevel::RK, Source/Advance.cpp:141-148; Source/Setup.cpp:194-196),
 *   - flux registers collect the RK-weighted face fluxes on both sides of each
 *     coarse-fine face and reflux the uncovered coarse cells
 *     (EBFluxRegister CrseAdd / FineAdd / Reflux, Source/Advance.cpp:344-360,
 *     Source/EBR.cpp:322-330),
 *   - covered coarse cells are replaced by the average of their fine cells
 *     (EB_average_down with unit volume fractions, Source/EBR.cpp:535-559),
 *   - the time step is the CFL bound over all levels (EBR::estTimeStep per
 *     level, dt_0 = min over levels of dt_l * 2^l, Source/EBR.cpp:240-305),
 *   - regridding tags cells with |d rho| >= refine_dengrad
 *     (Source/Tagging.H:11-36), buffers them by n_error_buf, clusters the
 *     tagged blocking_factor blocks into boxes no larger than max_grid_size and
 *     keeps every level properly nested in the one below.
 * Ideal-gas boxes, optionally cut by an embedded body (ocfd_amr_set_eb); one
 * CUDA graph launch per coarse step.                                          */
#define OCFD_AMR_MAX_LEVELS 6

typedef struct ocfd_amr ocfd_amr;

typedef struct ocfd_amr_desc {
    int32_t nbox0;               /* level-0 boxes (disjoint, covering the domain) */
    const ocfd_box* boxes0;
    ocfd_box domain;             /* level-0 domain */
    int32_t lo_bc[3], hi_bc[3];  /* ebr.lo_bc / ebr.hi_bc */
    double dx[3];                /* level-0 cell size */
    double prob_lo[3];
    int32_t bc_case;             /* OCFD_CASE_* */
    double case_params[16];
    int32_t max_level;           /* amr.max_level: finest level index allowed */
    int32_t blocking_factor[3];  /* amr.blocking_factor, in cells of the level built */
    int32_t max_grid_size[3];    /* amr.max_grid_size */
    int32_t n_error_buf;         /* amr.n_error_buf */
    int32_t regrid_int;          /* amr.regrid_int (coarse steps), 0 = never inside ocfd_amr_advance */
    double refine_dengrad;       /* ebr.refine_dengrad */
} ocfd_amr_desc;

ocfd_status ocfd_amr_create(ocfd_context* ctx, const ocfd_amr_desc* desc, ocfd_amr** amr);

/* A reacting hierarchy (the CHEM build's EBR::advance over subcycled levels,
 * Source/Advance.cpp:158-174, Source/CHEM/FlowAdvance.cpp:9-90, Source/EBR.cpp:
 * 313-357): 5 + 9 components per level (conserved state, then the partial
 * densities in the mechanism's order), on every level and substep
 *   chemistry over dt_l / 2 in iter_l substeps (iter_l = chem_substeps / 2^l on
 *   levels 0..2, 1 finer: the reference's 4 / 2^level), the multispecies flow
 *   step (RK2 by default, as the reference's flow_advance_multi; flux registers
 *   of the flow and of the species, flux_reg / flux_reg_spec), chemistry over
 *   dt_l / 2 again;
 * after the finer level's substeps: reflux of flow and species, species
 * renormalisation (clip, rescale to rho), average-down.  The coarse step is the
 * fixed `dt` (the CHEM build's fixed time step, Source/Advance.cpp:54-57), dt_l
 * = dt / 2^l.  Regridding tags on the density gradient as for the ideal gas.
 * No embedded body. */
typedef struct ocfd_amr_react_desc {
    double dt;                   /* coarse step (s) */
    int32_t chem_substeps;       /* substeps per half step on level 0 (the reference: 4) */
    uint32_t flags;              /* OCFD_VISC: mixture-averaged viscous and species transport;
                                    OCFD_FLUX_FP32: the mixed form of the face fluxes */
} ocfd_amr_react_desc;

ocfd_status ocfd_amr_create_reacting(ocfd_context* ctx, const ocfd_amr_desc* desc,
                                     const ocfd_amr_react_desc* react, ocfd_amr** amr);
/* Cut every level, present and future, with an embedded body (see
 * ocfd_level_set_eb): per box the regular, cut-cell or covered scheme of
 * EBR::compute_dSdt; cut-cell fluxes enter the flux registers weighted by their
 * area fractions and the reflux of a cut coarse cell is divided by its volume
 * fraction (EBFluxRegister with areafrac / volfrac, Source/Advance.cpp:344-360,
 * Source/EBR.cpp:322-330); average-down weights the fine cells by their volume
 * fractions (EB_average_down, Source/EBR.cpp:549-557); coarse-fine ghost cells
 * whose parent or a face neighbour of it is cut or covered are interpolated
 * piecewise-constant.  kind OCFD_EB_NONE removes the body.  Synchronous. */
ocfd_status ocfd_amr_set_eb(ocfd_amr* amr, const ocfd_eb_desc* eb);
/* Time integration of every level, present and future (orders as
 * ocfd_level_set_time_integration).  Under Heun and Euler the coarse-fine
 * ghosts of a fine stage at time t are AMReX FillPatch's linear interpolation
 * between the coarse old and new states (Source/Advance.cpp:119,126) and the
 * stage fluxes enter the flux registers with weight 0.5 dt (Heun) or dt
 * (Euler); under SSP-RK3 they come from the coarse stage states (above).
 * Synchronous. */
ocfd_status ocfd_amr_set_time_integration(ocfd_amr* amr, int32_t order);
/* ocfd_level_autotune for every level; the choice per level index is kept for
 * the levels later regrids build.  ocfd_amr_tuned reads a level's tile shape and
 * schedule (0 on success, -1 for a bad level). */
ocfd_status ocfd_amr_autotune(ocfd_amr* amr, unsigned flags, int reps, void* stream);
int ocfd_amr_tuned(const ocfd_amr* amr, int lev, int32_t* tile, int32_t* sched);
ocfd_status ocfd_amr_destroy(ocfd_amr* amr);
int ocfd_amr_nlevels(const ocfd_amr* amr);
/* The level object of level `lev` (state access through ocfd_level_state /
 * copy_in / copy_out); owned by the hierarchy, valid until the next regrid. */
ocfd_level* ocfd_amr_level(ocfd_amr* amr, int lev);
/* Boxes of level `lev`: writes min(cap, n) boxes and returns n (-1 on error). */
int ocfd_amr_get_grids(const ocfd_amr* amr, int lev, ocfd_box* out, int cap);
/* Tag levels lbase.. and rebuild the grids of levels lbase+1..max_level (data of
 * new cells interpolated from the level below, of old cells copied). Called with
 * lbase = finest level it adds one level (hierarchy construction at t = 0). */
ocfd_status ocfd_amr_regrid(ocfd_amr* amr, int lbase, void* stream);
/* Replace levels 1..nlev-1 by the given boxes (a recorded regrid replayed);
 * nbox[l] boxes of level l follow each other in `boxes`, level 1 first. */
ocfd_status ocfd_amr_set_grids(ocfd_amr* amr, int nlev, const int32_t* nbox, const ocfd_box* boxes,
                               void* stream);
/* Covered coarse cells := average of their fine cells, finest level first. */
ocfd_status ocfd_amr_average_down(ocfd_amr* amr, void* stream);
/* Ghost cells of every level at the current time (exchange, coarse-fine
 * interpolation, physical BCs). */
ocfd_status ocfd_amr_fill_ghosts(ocfd_amr* amr, void* stream);
/* nsteps coarse steps (regridding every regrid_int steps). */
ocfd_status ocfd_amr_advance(ocfd_amr* amr, int nsteps, double cfl, unsigned flags, void* stream);
ocfd_status ocfd_amr_time(ocfd_amr* amr, double* time, double* last_dt0, void* stream);
ocfd_status ocfd_amr_set_time(ocfd_amr* amr, double time, void* stream);
ocfd_status ocfd_amr_set_stop_time(ocfd_amr* amr, double stop_time, void* stream);
/* Cell-steps of one coarse step: leaf = cells not covered by a finer level,
 * all = every cell advanced; each weighted by the level's 2^lev substeps. */
ocfd_status ocfd_amr_cell_steps(const ocfd_amr* amr, int64_t* leaf, int64_t* all);
/* State FABs of level `lev` (grown boxes back to back, layout of
 * ocfd_level_copy_in) to / from host or device memory; the hierarchy's clock is
 * left alone.  ocfd_amr_state_elems gives the number of doubles. */
size_t ocfd_amr_state_elems(const ocfd_amr* amr, int lev);
ocfd_status ocfd_amr_copy_in(ocfd_amr* amr, int lev, const double* buf, void* stream);
ocfd_status ocfd_amr_copy_out(ocfd_amr* amr, int lev, double* buf, void* stream);
/* The valid cells of level `lev` only (layout of ocfd_level_copy_valid_in,
 * ocfd_amr_valid_elems doubles); the hierarchy's clock is left alone. */
int64_t ocfd_amr_valid_elems(const ocfd_amr* amr, int lev);
ocfd_status ocfd_amr_copy_valid_in(ocfd_amr* amr, int lev, const double* buf, void* stream);
ocfd_status ocfd_amr_copy_valid_out(ocfd_amr* amr, int lev, double* buf, void* stream);
/* Plotfile of the hierarchy's current state: rho, xmom, ymom, zmom, Eden (the
 * state names of Source/Setup.cpp:202-206) and the derived ux, uy, uz and
 * pressure (Source/Setup.cpp:95-110, 164-178); level steps step * 2^lev. */
ocfd_status ocfd_amr_write_plotfile(ocfd_amr* amr, const char* dir, int32_t step, void* stream);
/* Kernel launches of one coarse step (the captured graph; memset / copy nodes
 * not counted). */
int ocfd_amr_launches_per_step(const ocfd_amr* amr);
/* Kernels launched by the hierarchy since its creation: graph launches times
 * their kernels, plus regridding, ghost filling and time-step estimation. */
int64_t ocfd_amr_kernels_launched(const ocfd_amr* amr);

/* ------------------------------------------------ plotfiles and comparison
 * AMReX plotfile layout (HyperCLaw-V1.1: Header, Level_<l>/Cell_H, Cell_D_00000
 * with one little-endian double FAB per box), the files AmrLevel::writePlotFile
 * writes for the reference (Source/IO.cpp:32-35), and the comparison of
 * Util/Plotfile/fcompare.cpp:150-290.  Host code; needs no device.            */
typedef struct ocfd_plot_level {
    int32_t nbox;
    const ocfd_box* boxes;       /* valid boxes of the level */
    const double* const* fabs;   /* per box: ncomp components over the box, i fastest, component slowest */
    double dx[3];
    int32_t step;                /* steps taken by the level */
} ocfd_plot_level;

ocfd_status ocfd_plotfile_write(const char* dir, int32_t nlev, const ocfd_plot_level* levels, int32_t ncomp,
                                const char* const* names, const ocfd_box* domain0, const double prob_lo[3],
                                const double prob_hi[3], int32_t ref_ratio, double time);
/* Levels and variables of a plotfile. */
ocfd_status ocfd_plotfile_info(const char* file, int32_t* nlev, int32_t* ncomp);
/* fcompare: per level l and variable n (index l * ncomp + n, up to cap entries)
 * the absolute error ||b - a|| (norm 0: max; 1 / 2: discrete L1 / L2 times
 * dV^(1/norm)) and the relative error ||b - a|| / ||a||; nan_flags bit 0 / 1 =
 * NaN in a / b.  allow_diff_grids compares over a's boxes. */
ocfd_status ocfd_plotfile_compare(const char* file_a, const char* file_b, int32_t norm, int32_t allow_diff_grids,
                                  int32_t cap, double* abs_err, double* rel_err, int32_t* nan_flags,
                                  int32_t* nlev, int32_t* ncomp);

/* ------------------------------------------- 5th-generation tensor cores
 * C[128 x N] = A[128 x K] * B[N x K]^T with row-major BF16 A and B (device),
 * FP32 C, on tcgen05.mma with the accumulator in tensor memory: the building
 * block of the chemistry surrogate's kernels, exposed for testing.  N and K in
 * [16, 256], multiples of 16.  Synchronises `stream`; OCFD_TIMEOUT if the
 * bounded wait for the MMA ran out. */
ocfd_status ocfd_tc_gemm_bf16(ocfd_context* ctx, const uint16_t* A, const uint16_t* B, float* C, int N, int K,
                              void* stream);

/* ------------------------------------------------ chemistry surrogate network
 * MLP 12 -> 128 x 4 (GELU) -> 10 on the tensor cores: BF16 weights and
 * activations, FP32 accumulation (tcgen05.mma into tensor memory).  Inputs
 * (T, ln p, sqrt of the 9 Y, log10 dt) and outputs (rates of T and of the 9 Y)
 * are used normalised: x_n = (x - in_mu) * in_isd, y = y_n * out_sd + out_mu.
 * Weights: five row-major (out x in) blocks W1 128x16 (inputs padded from 12),
 * W2..W4 128x128, W5 16x128 (outputs padded from 10), 53248 floats; biases
 * 128 x 4 + 16 = 528 floats.                                                    */
typedef struct ocfd_mlp ocfd_mlp;
#define OCFD_MLP_WEIGHTS 53248
#define OCFD_MLP_BIASES 528

/* He-normal initial weights from `seed`; training batches up to max_batch rows
 * (a multiple of 256). */
ocfd_status ocfd_mlp_create(ocfd_context* ctx, int32_t max_batch, uint64_t seed, ocfd_mlp** mlp);
ocfd_status ocfd_mlp_destroy(ocfd_mlp* mlp);
ocfd_status ocfd_mlp_set_norm(ocfd_mlp* mlp, const float in_mu[12], const float in_isd[12], const float out_mu[10],
                              const float out_sd[10]);
/* Outputs as signed logarithms of rates: with scale[k] > 0 the network's output
 * y_k (after out_mu / out_sd) stands for the rate sign(y) scale[k] expm1(|y|),
 * and an increment over dt is rate * dt (0: y is the rate itself). */
ocfd_status ocfd_mlp_set_target_scale(ocfd_mlp* mlp, const float scale[10]);
/* FP32 master parameters (host arrays of OCFD_MLP_WEIGHTS / OCFD_MLP_BIASES). */
ocfd_status ocfd_mlp_get_params(ocfd_mlp* mlp, float* W, float* b);
ocfd_status ocfd_mlp_set_params(ocfd_mlp* mlp, const float* W, const float* b);
/* Y [M x 10] = network(X [M x 12]), normalised units, device arrays, M a
 * multiple of 128 up to max_batch. */
ocfd_status ocfd_mlp_forward(ocfd_mlp* mlp, const float* X, float* Y, int64_t M, void* stream);
/* One step on normalised device batches X [M x 12], T [M x 10]: forward, mean
 * squared error, backward, and with `update` an Adam step of rate lr; the loss
 * and (optional, host) gradients gW [OCFD_MLP_WEIGHTS], gb [OCFD_MLP_BIASES]. */
ocfd_status ocfd_mlp_train_step(ocfd_mlp* mlp, const float* X, const float* T, int64_t M, float lr, int32_t update,
                                float* loss, float* gW, float* gb, void* stream);

/* Guard of the surrogate chemistry substep: a cell takes the network's increments
 * only when its inputs lie in the training range and the increments keep every
 * Y in [-y_tol, 1 + y_tol] and the H, O, N element contents within elem_tol
 * (relative), and, when dy_rel_max > 0, change no Y_n by more than
 * dy_rel_max * max(Y_n, y_floor) (the per-output error criterion); otherwise
 * the FP64 implicit substep is applied to it. */
typedef struct ocfd_surrogate_guard {
    double T_min, T_max, p_min, p_max, dt_min, dt_max;
    double y_tol, elem_tol;
    double dy_rel_max, y_floor;
} ocfd_surrogate_guard;

/* Chemistry of a reacting level by the network (NULL: back to the FP64
 * substep): every substep runs the network over the level's cells and the FP64
 * substep over the cells its guard rejected.  ocfd_react_fallbacks: cells sent
 * to the FP64 substep so far. */
ocfd_status ocfd_react_set_surrogate(ocfd_react* react, ocfd_mlp* mlp, const ocfd_surrogate_guard* guard);
ocfd_status ocfd_react_fallbacks(ocfd_react* react, int64_t* fallbacks, void* stream);

/* 0D cells: n states of 14 components (component stride n, device memory). */
/* one FP64 implicit substep per cell, step dt_cells[i] (or dt when NULL) */
ocfd_status ocfd_chem_cells_advance(ocfd_context* ctx, int64_t n, double* U, const double* dt_cells, double dt,
                                    void* stream);
/* T, p, Y[9] of each cell into out [11][n] */
ocfd_status ocfd_chem_cells_props(ocfd_context* ctx, int64_t n, const double* U, double* out, void* stream);
/* constant-pressure restoration after a constant-volume substep: each cell at
 * rest is brought to p_target[i] (device, n doubles) at the enthalpy
 * e + p_target / rho (mass fractions kept); the generator of constant-pressure
 * ignition states.  No counterpart in the reference. */
ocfd_status ocfd_chem_cells_isobaric(ocfd_context* ctx, int64_t n, double* U, const double* p_target, void* stream);
/* one surrogate substep of dt per cell (with the FP64 fallback); *fallbacks
 * receives the number of cells the guard sent to the FP64 substep */
ocfd_status ocfd_chem_cells_surrogate(ocfd_context* ctx, ocfd_mlp* mlp, const ocfd_surrogate_guard* guard,
                                      int64_t n, double* U, double dt, int64_t* fallbacks, void* stream);

/* ----------------------------------------------------------- measurement */
/* Sustained FP64 and FP32 FMA rates of the current device in GFLOP/s (2 flops
 * per FMA), from register-only FMA chains over all SMs. */
ocfd_status ocfd_measure_fma_peaks(double* fp64_gflops, double* fp32_gflops);

/* Packed FP32 FMA rate (FFMA2: two lanes per instruction) of the current device
 * in GFLOP/s (4 flops per instruction); the FP32 denominator of the mixed form,
 * whose WENO-Z runs on packed pairs.  No counterpart in the reference. */
ocfd_status ocfd_measure_ffma2_peak(double* fp32x2_gflops);

/* Test hook: the FP32-flux form stages the cross of each tile of depth >= 4
 * (the tile and its +-3 halos along x, y and z) by TMA (on != 0, the default)
 * or with plain loads (0), in stage tables built from now on; both give the
 * same results.  No counterpart in the reference. */
void ocfd_set_tma_staging(int32_t on);

/* Test hook: fast[i] = the reciprocal the fused FP64 kernels use in place of an
 * IEEE division (approximate seed + two Newton-Raphson steps), ieee[i] = 1/x[i]
 * correctly rounded; device arrays of n doubles.  No counterpart in the
 * reference. */
ocfd_status ocfd_check_rcp_f64(const double* x, double* fast, double* ieee, int64_t n, void* stream);

#ifdef __cplusplus
}
#endif
#endif
