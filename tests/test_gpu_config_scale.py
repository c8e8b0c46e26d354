"""Parity at the benchmark configurations' own sizes and step counts: the GPU's
plain FP64 form against the oracle (OpenMP build) on the same inputs.

* Sod shock tube 512x64x4 (a thin 2D slab), 200 SSP-RK3 steps at CFL 0.5;
* double Mach reflection, base level 1024x256x2, 200 SSP-RK3 steps at CFL 0.5;
* the double Mach reflection hierarchy (2 refined levels, ratio 2, |d rho| >= 0.05
  tagging, blocking factor 32, max grid 128, regrid every 2 coarse steps) on a
  256x64x2 base - a quarter of the benchmark's base in each direction, so that the
  CPU restatement of the hierarchy finishes in about a minute - for 20 coarse
  steps with its regrids;
* the 3D H2/air reacting box (9 species, Li-Dryer, viscous, 8 hot spots of
  peak 1800 K, radius 6 cells, dx = 78 um): a 64^3 sample of the 128^3 box for
  100 Strang steps of the reference's sequence (4 chemistry substeps over dt/2,
  RK2 flow step, 4 substeps, renormalisation; Source/Advance.cpp:158-174,
  Source/CHEM/FlowAdvance.cpp:9-90), dt = 1e-8 s.

For each: the RHS of one evaluation, GPU against oracle, on the initial and on
the final state, within 1e-12 norm-wise (the reacting box starts at rest, so its
right-hand side is measured against the split-flux scale, see rhs_err); after N
steps the two final states within 1e-10 (grouped max norm; 1e-9 for the 9
species of the reacting box, whose radicals start at zero), and their L1 errors (fcompare's
sum|a-b| / sum|b|) in density, pressure and, for the reacting box, Y_OH and
Y_H2O within 1e-10 of each other; Sod's L1 error against the exact Riemann
solution is the same for both to 1e-10 relative.
"""
import numpy as np
import pytest

from test_gpu_level import oracle_bc, relerr, valid

pytestmark = pytest.mark.gpu

NG = 4
GAMMA = 1.4


@pytest.fixture(scope="module")
def ctx():
    import ocfd
    return ocfd.Context()


def l1(a, b):
    """fcompare's relative L1 norm of a - b (uniform cells)"""
    return float(np.abs(a - b).sum() / np.abs(b).sum())


def pressure(U):
    return (GAMMA - 1.0) * (U[4] - 0.5 * (U[1] ** 2 + U[2] ** 2 + U[3] ** 2) / U[0])


def rhs_parity(ctx, oracle, case, G):
    """RHS of the ghost-filled grown state G (whole domain as one box): GPU
    against the oracle; returns the grouped relative error."""
    import torch
    S = np.ascontiguousarray(G.copy())
    oracle.fill_ghosts(oracle_bc(case), S)
    n = case["n"]
    dxinv = [1.0 / x for x in case["dx"]]
    ref, _ = oracle.rhs_regular(S, dxinv)
    St = torch.from_numpy(S).cuda()
    dS = torch.empty((5, n[2], n[1], n[0]), dtype=torch.float64, device="cuda")
    ctx.rhs_regular_box(St, dS, (0, 0, 0), tuple(x - 1 for x in n), dxinv)
    torch.cuda.synchronize()
    return relerr(dS.cpu().numpy(), ref)


def run_both(ctx, oracle_omp, case, steps, max_grid):
    from test_gpu_level import run_gpu
    S = np.ascontiguousarray(case["G"].copy())
    tr, _ = oracle_omp.advance_rk3(oracle_bc(case), S, 0.5, steps, form=1)
    got, tg = run_gpu(ctx, case, steps, 0.5, max_grid)
    return got, tg, S, tr


def grown(case, V):
    G = np.zeros_like(case["G"])
    G[:, NG:-NG, NG:-NG, NG:-NG] = V
    return G


def test_sod_512x64x4_200_steps(ctx, oracle, oracle_omp):
    from exact_riemann import sample
    from ocfd.cases import sod
    case = sod(512, 64, 4)
    assert rhs_parity(ctx, oracle, case, case["G"]) <= 1e-12
    got, tg, S, tr = run_both(ctx, oracle_omp, case, 200, (128, 64, 4))
    ref = valid(S)
    assert tg == pytest.approx(tr, rel=1e-13)
    assert relerr(got, ref) <= 1e-10
    assert rhs_parity(ctx, oracle, case, S) <= 1e-12
    for f in (lambda U: U[0], pressure):
        assert l1(f(got), f(ref)) <= 1e-10
    # L1 error against the exact solution at the final time, the same for both
    x = (np.arange(512) + 0.5) / 512
    ex = sample(x, tr, 0.5, (1.0, 0.0, 1.0), (0.125, 0.0, 0.1))
    err = []
    for U in (got, ref):
        e_rho = np.abs(U[0] - ex[0][None, None, :]).mean()
        e_p = np.abs(pressure(U) - ex[2][None, None, :]).mean()
        err.append((e_rho, e_p))
    assert 0.0 < err[1][0] < 5e-3 and 0.0 < err[1][1] < 5e-3   # a converging scheme at t ~ 0.2
    for a, b in zip(*err):
        assert abs(a - b) <= 1e-10 * b


def test_dmr_base_1024x256x2_200_steps(ctx, oracle, oracle_omp):
    from ocfd.cases import dmr
    case = dmr(1024, 256, 2)
    assert rhs_parity(ctx, oracle, case, case["G"]) <= 1e-12
    got, tg, S, tr = run_both(ctx, oracle_omp, case, 200, (128, 128, 2))
    ref = valid(S)
    assert tg == pytest.approx(tr, rel=1e-13)
    assert relerr(got, ref) <= 1e-10
    assert rhs_parity(ctx, oracle, case, S) <= 1e-12
    for f in (lambda U: U[0], pressure):
        assert l1(f(got), f(ref)) <= 1e-10


def test_dmr_hierarchy_20_coarse_steps(ctx, oracle_omp):
    from ocfd.cases import dmr_amr
    from ocfd.level import chop_domain
    from test_gpu_amr import compare_levels, make_hierarchy, make_oracle, oracle_build
    case = dmr_amr(256, 64, 2, max_level=2, blocking_factor=32, max_grid=128, n_error_buf=1,
                   refine_dengrad=0.05, regrid_int=2)
    case["boxes0"] = chop_domain(case["n"], case["max_grid_size"])
    H = make_hierarchy(ctx, case)
    H.build(case["fab"])
    A = make_oracle(oracle_omp, case)
    oracle_build(A, case["fab"])
    compare_levels(H, A, 1e-15)
    for step in range(20):
        if step > 0 and step % case["regrid_int"] == 0:
            A.regrid(0)
        A.step(0.5)
        H.advance(1, 0.5)
        if step % 5 == 4:
            t, _ = H.time()
            assert abs(t - A.time) <= 1e-13 * A.time
            compare_levels(H, A, 1e-10)
    assert H.nlevels() == 3
    # L1 of density and pressure on every level, GPU against the restatement
    for lev in range(H.nlevels()):
        g, m = H.level_global(lev)
        o, _ = A.valid(lev)
        G, O = g[:, m], o[:, m]
        assert l1(G[0], O[0]) <= 1e-10
        assert l1(pressure(G), pressure(O)) <= 1e-10
    H.close()


def test_react_64cube_sample_100_steps(ctx, oracle, oracle_omp):
    import torch
    from ocfd.cases import react_cube
    from ocfd.level import chop_domain
    from test_gpu_react import oracle_step, run_gpu
    case = react_cube(ctx, n=64, length=0.01 * 64 / 128)
    n = 64
    dxinv = [1.0 / x for x in case["dx"]]

    def filled(G):
        """conserved state and partial densities with periodic ghosts"""
        from oracle import BCStruct
        S = np.ascontiguousarray(G[:5].copy())
        sp = np.ascontiguousarray(G[5:].copy())
        bc = BCStruct()
        bc.lo_bc[:] = [0, 0, 0]; bc.hi_bc[:] = [0, 0, 0]
        bc.dx[:] = list(case["dx"]); bc.dom_hi[:] = [n - 1] * 3
        oracle.fill_ghosts(bc, S)
        oracle.fill_ghosts(bc, sp)
        return S, sp

    def pressure_of(V):
        S, sp = filled(grown(dict(G=case["G"]), V))
        return oracle_omp.c2prim(S, sp)[4, NG:-NG, NG:-NG, NG:-NG]

    def rhs_err(G):
        """The box starts at rest at uniform pressure, so every component of its
        right-hand side is the small difference of split fluxes of size rho c
        (mass, species), rho c^2 (momentum) and rho c H (energy); the error of
        each is measured against dxinv times that flux scale (norm-wise over
        the box) rather than against the residual itself."""
        S, sp = filled(G)
        rS, rsp, *_ = oracle_omp.rhs_chem(S, sp, dxinv, do_visc=True)
        dS = torch.empty((5, n, n, n), dtype=torch.float64, device="cuda")
        dsp = torch.empty((9, n, n, n), dtype=torch.float64, device="cuda")
        ctx.rhs_chem_box(torch.from_numpy(S).cuda(), torch.from_numpy(sp).cuda(), dS, dsp, (0, 0, 0),
                         (n - 1,) * 3, dxinv, flags=1)
        torch.cuda.synchronize()
        q = oracle_omp.c2prim(S, sp)[:, NG:-NG, NG:-NG, NG:-NG]
        rho, p, c = q[0], q[4], q[6]
        H = np.abs(S[4, NG:-NG, NG:-NG, NG:-NG]) / rho + p / rho
        scale = max(dxinv) * np.array([(rho * c).max(), (rho * c * c).max(), (rho * c * H).max()])
        g, r = dS.cpu().numpy(), rS
        err = max(np.abs(g[0] - r[0]).max() / scale[0], np.abs(g[1:4] - r[1:4]).max() / scale[1],
                  np.abs(g[4] - r[4]).max() / scale[2],
                  np.abs(dsp.cpu().numpy() - rsp).max() / scale[0])
        return err

    def state_err(a, b):
        """grouped max-norm error of two states; momentum against rho c (the box
        is nearly at rest, so momentum itself is a small residual)"""
        q = oracle_omp.c2prim(*filled(grown(dict(G=case["G"]), b)))[:, NG:-NG, NG:-NG, NG:-NG]
        e = max(np.abs(a[0] - b[0]).max() / np.abs(b[0]).max(), np.abs(a[4] - b[4]).max() / np.abs(b[4]).max(),
                np.abs(a[1:4] - b[1:4]).max() / (q[0] * q[6]).max())
        for s in range(5, 14):
            e = max(e, np.abs(a[s] - b[s]).max() / max(np.abs(b[s]).max(), 1e-300))
        return e

    assert rhs_err(case["G"]) <= 1e-12
    S = np.ascontiguousarray(case["G"][:5].copy())
    sp = np.ascontiguousarray(case["G"][5:].copy())
    steps = 100
    for _ in range(steps):
        oracle_step(oracle_omp, S, sp, case["dx"], 1e-8, 2, 4)
    want = np.concatenate([S, sp])[:, NG:-NG, NG:-NG, NG:-NG]
    got = run_gpu(ctx, case, chop_domain(case["n"], 32), steps, 2)
    assert state_err(got, want) <= 1e-9
    assert rhs_err(grown(dict(G=case["G"]), want)) <= 1e-12
    # L1 in density, pressure, Y_OH and Y_H2O (species order H2 O2 H2O H O OH HO2 H2O2 N2)
    assert l1(got[0], want[0]) <= 1e-10
    assert l1(pressure_of(got), pressure_of(want)) <= 1e-10
    for s in (5, 2):
        assert l1(got[5 + s] / got[0], want[5 + s] / want[0]) <= 1e-10
    # the chemistry ran: OH and water grew in the hot spots
    assert (want[5 + 5] / want[0]).max() > 1e-8
