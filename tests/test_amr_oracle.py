"""The CPU restatement of the AMR hierarchy (oracle/amr_oracle.py) checked on
its own before it serves as the GPU path's checker: reflux makes the composite
step conservative, the coarse-fine interpolation is exact on linear data and
conservative, the time interpolation reproduces the coarse RK3 stages, and a
uniform state stays uniform on three levels."""
import numpy as np
import pytest

from amr_oracle import AmrOracle, mix_coefs

NG = 4


def chop(n, m):
    out = []
    for z in range(0, n[2], m):
        for y in range(0, n[1], m):
            for x in range(0, n[0], m):
                out.append(((x, y, z), (min(x + m, n[0]) - 1, min(y + m, n[1]) - 1, min(z + m, n[2]) - 1)))
    return out


def pulse_fab(lev, lo, hi, d):
    x = (np.arange(lo[0] - NG, hi[0] + NG + 1) + 0.5) * d[0]
    y = (np.arange(lo[1] - NG, hi[1] + NG + 1) + 0.5) * d[1]
    z = (np.arange(lo[2] - NG, hi[2] + NG + 1) + 0.5) * d[2]
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    rho = 1.0 + 0.5 * np.exp(-((X - 0.5) ** 2 + (Y - 0.25) ** 2 + (Z - 0.125) ** 2) / 0.01)
    u, v, w, p = 1.0, 0.5, 0.25, 1.0
    return np.stack([rho, rho * u, rho * v, rho * w, p / 0.4 + 0.5 * rho * (u * u + v * v + w * w)])


def test_time_interpolation_weights():
    # weights sum to one; stage 1 of the first fine substep is u0; the end of
    # the second substep is the coarse end state U3 = D
    for kind in range(4):
        for th in (0.0, 0.5):
            assert sum(mix_coefs(kind, th)) == pytest.approx(1.0, abs=1e-15)
    assert mix_coefs(0, 0.0) == (1.0, 0.0, 0.0, 0.0)
    a = mix_coefs(3, 0.5)
    assert a == pytest.approx((0.0, 0.0, 0.0, 1.0), abs=1e-15)
    # linear ODE u' = lam u: fine stage values from the coarse stages equal the
    # fine RK3 stage states of the same ODE to O(h^3)
    lam, dt = -0.7, 0.1
    u0 = 1.0
    U1 = u0 + dt * lam * u0
    U2 = 0.75 * u0 + 0.25 * (U1 + dt * lam * U1)
    U3 = u0 / 3 + 2.0 / 3.0 * (U2 + dt * lam * U2)
    h = dt / 2
    f1 = u0 + h * lam * u0
    f2 = 0.75 * u0 + 0.25 * (f1 + h * lam * f1)
    for kind, want in ((0, u0), (1, f1), (2, f2)):
        a = mix_coefs(kind, 0.0)
        got = a[0] * u0 + a[1] * U1 + a[2] * U2 + a[3] * U3
        assert abs(got - want) < 5 * (abs(lam) * h) ** 3


def periodic_oracle(orc, max_level=1, time_integration=3):
    n = (32, 16, 8)
    dx = 1.0 / 32
    A = AmrOracle(orc, n, (dx,) * 3, (0, 0, 0), (0, 0, 0), chop(n, 16), max_level=max_level,
                  blocking_factor=(8, 8, 8), max_grid_size=(16, 16, 16), time_integration=time_integration)
    A.set_level_fabs(0, pulse_fab)
    A.fill_all_sync()
    return A


@pytest.mark.parametrize("order", [3, 2, 1])
def test_reflux_conserves(oracle, order):
    """composite conservation under every time integration: the flux registers
    take each stage's fluxes with the scheme's weights (RK3 1/6, 1/6, 2/3; RK2
    1/2, 1/2; Euler 1)"""
    A = periodic_oracle(oracle, time_integration=order)
    A.apply_grids(0, [[((16, 8, 4), (39, 23, 11)), ((56, 0, 0), (63, 15, 15))]])
    A.average_down_all()
    V, m = A.valid(0)
    s0 = V[:, m].sum(axis=1)
    for _ in range(3):
        A.step(0.5)
    V, m = A.valid(0)
    s1 = V[:, m].sum(axis=1)
    assert (np.abs(s1 - s0) / np.abs(s0)).max() < 1e-13


def test_interpolation_linear_and_conservative(oracle):
    n = (16, 16, 16)
    dx = 1.0 / 16
    g = np.array([0.3, -0.2, 0.1])

    def fab(lev, lo, hi, d):
        x = (np.arange(lo[0] - NG, hi[0] + NG + 1) + 0.5) * d[0]
        y = (np.arange(lo[1] - NG, hi[1] + NG + 1) + 0.5) * d[1]
        z = (np.arange(lo[2] - NG, hi[2] + NG + 1) + 0.5) * d[2]
        Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
        lin = 1.0 + g[0] * X + g[1] * Y + g[2] * Z
        return np.stack([lin, 2 * lin, -lin, 0.5 * lin, 3 * lin])
    A = AmrOracle(oracle, n, (dx,) * 3, (2, 2, 2), (2, 2, 2), chop(n, 16), max_level=1,
                  blocking_factor=(8, 8, 8), max_grid_size=(16, 16, 16))
    A.set_level_fabs(0, fab)
    A.fill_all_sync()
    fine = [((8, 8, 8), (23, 23, 23))]
    A.apply_grids(0, [fine])
    got = A.levels[1]["U"]
    want = fab(1, (0, 0, 0), (31, 31, 31), A.dx(1))
    sl = (slice(None), slice(8, 8 + 16 + 2 * NG), slice(8, 8 + 16 + 2 * NG), slice(8, 8 + 16 + 2 * NG))
    assert np.abs(got[sl] - want[sl]).max() < 1e-14
    # conservative: averaging the new fine cells back gives the coarse values
    # (also on non-linear data, where the limiter is active)
    A.set_level_fabs(0, pulse_fab)
    A.fill_all_sync()
    A.levels = A.levels[:1]
    A.apply_grids(0, [fine])
    c = A.levels[0]["U"][:, NG:-NG, NG:-NG, NG:-NG].copy()
    A.average_down_all()
    assert np.abs(A.levels[0]["U"][:, NG:-NG, NG:-NG, NG:-NG] - c).max() < 1e-14


@pytest.mark.parametrize("order", [3, 2, 1])
def test_free_stream_three_levels(oracle, order):
    """a uniform state stays uniform on three subcycled levels under every time
    integration (the coarse-fine ghosts of each scheme's stages reproduce it)"""
    A = periodic_oracle(oracle, max_level=2, time_integration=order)
    st = np.array([1.3, 0.91, -0.52, 0.26, 5.9])

    def fab(lev, lo, hi, d):
        shape = (hi[2] - lo[2] + 1 + 2 * NG, hi[1] - lo[1] + 1 + 2 * NG, hi[0] - lo[0] + 1 + 2 * NG)
        return np.stack([np.full(shape, s) for s in st])
    A.set_level_fabs(0, fab)
    A.fill_all_sync()
    A.apply_grids(0, [[((16, 8, 0), (47, 23, 15))], [((40, 24, 8), (87, 39, 23))]])
    for _ in range(3):
        A.step(0.5)
    for l in range(3):
        V, m = A.valid(l)
        assert np.abs(V[:, m] - st[:, None]).max() < 1e-13 * np.abs(st).max()


def test_regrid_tags_and_nests(oracle):
    """grids made from density-gradient tags cover every tagged cell and each
    level is nested in the one below by two coarse cells"""
    import sys
    import os
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "opencfd-amr_gb300"))
    from ocfd.cases import dmr_amr
    case = dmr_amr(nx=64, ny=16, nz=2, max_level=2, blocking_factor=8, max_grid=16)
    A = AmrOracle(oracle, case["n"], case["dx"], case["lo_bc"], case["hi_bc"], chop(case["n"], 16),
                  case["prob_lo"], case["bc_case"], case["case_params"], 2, case["blocking_factor"],
                  case["max_grid_size"], case["n_error_buf"], case["refine_dengrad"])
    A.set_level_fabs(0, case["fab"])
    A.regrid(0)
    A.set_level_fabs(1, case["fab"])
    A.regrid(1)
    assert len(A.levels) == 3
    for l in range(2):
        A.fill_all_sync()
        U = A.levels[l]["U"][0]
        c = U[NG:-NG, NG:-NG, NG:-NG]
        fine = A.levels[l + 1]["mask"]
        cov = fine.reshape(fine.shape[0] // 2, 2, fine.shape[1] // 2, 2, fine.shape[2] // 2, 2).any(axis=(1, 3, 5))
        gx = np.maximum(np.abs(U[NG:-NG, NG:-NG, NG + 1:U.shape[2] - NG + 1] - c),
                        np.abs(c - U[NG:-NG, NG:-NG, NG - 1:U.shape[2] - NG - 1]))
        gy = np.maximum(np.abs(U[NG:-NG, NG + 1:U.shape[1] - NG + 1, NG:-NG] - c),
                        np.abs(c - U[NG:-NG, NG - 1:U.shape[1] - NG - 1, NG:-NG]))
        tagged = (np.maximum(gx, gy) >= 0.05) & A.levels[l]["mask"]
        assert tagged.any()
        if l == 0:
            assert cov[tagged].all()
        # nesting: every fine box coarsened and grown by 2 lies in level l (or outside the domain)
        below = A.levels[l]["mask"]
        for lo, hi in A.levels[l + 1]["boxes"]:
            clo = [max(v // 2 - 2, 0) for v in lo]
            chi = [min(v // 2 + 2, below.shape[2 - d] - 1) for d, v in enumerate(hi)]
            assert below[clo[2]:chi[2] + 1, clo[1]:chi[1] + 1, clo[0]:chi[0] + 1].all()
        for lo, hi in A.levels[l + 1]["boxes"]:
            for d in range(3):
                ext = hi[d] - lo[d] + 1
                assert ext <= 16 and lo[d] % min(8, A.n(l + 1)[d]) == 0


def test_cut_cell_operators_with_the_body(oracle):
    """The restatement with an embedded cylinder (the checker of the GPU's cut
    hierarchy), on its own: box classes follow the geometry, the
    volume-fraction average-down of a uniform fine level is that uniform state
    (and the plain average where nothing is cut), and two coarse steps of the
    jet past the cylinder stay finite with positive density and energy."""
    from amr_oracle import BOX_CUT, BOX_REGULAR
    from ocfd.cases import jet_eb_amr

    case = jet_eb_amr(nx=64, ny=32, nz=4, max_level=2, blocking_factor=8, max_grid=16, n_error_buf=1,
                      refine_dengrad=0.1, regrid_int=2)
    boxes0 = chop(case["n"], 16)
    A = AmrOracle(oracle, case["n"], case["dx"], case["lo_bc"], case["hi_bc"], boxes0, case["prob_lo"],
                  case["bc_case"], case["case_params"], case["max_level"], case["blocking_factor"],
                  case["max_grid_size"], case["n_error_buf"], case["refine_dengrad"], eb=case["eb"])
    A.set_level_fabs(0, case["fab"])
    for lev in range(A.max_level):
        if len(A.levels) != lev + 1:
            break
        A.regrid(lev)
        if len(A.levels) == lev + 2:
            A.set_level_fabs(lev + 1, case["fab"])
    A.average_down_all()
    assert len(A.levels) == 3
    cls0 = A.classes(0)
    assert BOX_CUT in cls0 and BOX_REGULAR in cls0
    # boxes far from the cylinder (more than 4 + 1 cells) are regular
    c = np.array(case["eb"]["center"]) / case["dx"][0]
    r = case["eb"]["radius"] / case["dx"][0]
    for cl, (lo, hi) in zip(cls0, A.levels[0]["boxes"]):
        near = [max(lo[d] - 5 - c[d], c[d] - (hi[d] + 6), 0.0) for d in (0, 1)]
        if np.hypot(*near) > r:
            assert cl == BOX_REGULAR
    # average-down of a uniform fine state is that state wherever a child is fluid
    F = A.levels[1]
    keep = F["U"].copy()
    F["U"][:] = 3.25
    D = A.levels[0]["U"].copy()
    A._avg_down(0, D)
    cov = A._covered(0)
    assert np.allclose(D[:, NG:-NG, NG:-NG, NG:-NG][:, cov], 3.25, rtol=1e-15)
    F["U"][:] = keep
    for _ in range(2):
        A.step(0.5)
    for l in range(len(A.levels)):
        V, m = A.valid(l)
        assert np.isfinite(V[:, m]).all() and V[0][m].min() > 0 and V[4][m].min() > 0


@pytest.mark.parametrize("order", [1, 2])
def test_time_integration_single_level_matches_box_restatement(oracle, order):
    """ebr.time_integration = RK2 (the reference's default) and Euler: the
    hierarchy restatement on one level of eight boxes against the single-box C
    restatement of Source/Advance.cpp:115-138 on the same periodic pulse"""
    from oracle import BCStruct
    n = (32, 16, 8)
    dx = 1.0 / 32
    A = periodic_oracle(oracle, max_level=0, time_integration=order)
    S = np.ascontiguousarray(pulse_fab(0, (0, 0, 0), (n[0] - 1, n[1] - 1, n[2] - 1), (dx,) * 3))
    bc = BCStruct()
    bc.lo_bc[:] = [0, 0, 0]
    bc.hi_bc[:] = [0, 0, 0]
    bc.dx[:] = [dx] * 3
    bc.dom_lo[:] = [0, 0, 0]
    bc.dom_hi[:] = [n[0] - 1, n[1] - 1, n[2] - 1]
    t, _ = oracle.advance_rk(bc, S, 0.5, 3, order)
    for _ in range(3):
        A.step(0.5)
    V, m = A.valid(0)
    assert m.all()
    assert A.time == pytest.approx(t, rel=1e-14)
    ref = S[:, NG:-NG, NG:-NG, NG:-NG]
    assert np.abs(V - ref).max() <= 1e-13 * np.abs(ref).max()


def test_reacting_restatement_conserves_mass_and_renormalises(oracle):
    """The reacting hierarchy restatement on a periodic box with one hot spot,
    two levels: total mass (level 0 after average-down) is conserved through
    chemistry, the RK2 flow step and reflux, and every cell's partial densities
    sum to its density after the step (the renormalisation)"""
    from amr_oracle import AmrOracle
    from inputs import react_hot_spot_fab
    from ocfd.level import chop_domain
    n0 = (8, 8, 8)
    dx = 7.8125e-5
    fab = react_hot_spot_fab(oracle, n0, dx, radius_cells=1.5)
    A = AmrOracle(oracle, n0, (dx,) * 3, (0, 0, 0), (0, 0, 0), chop_domain(n0, (8, 8, 8)), max_level=1,
                  blocking_factor=(4, 4, 4), max_grid_size=(8, 8, 8), n_error_buf=1, refine_dengrad=0.002,
                  react=dict(dt=1e-8, chem_substeps=4, visc=True))
    A.set_level_fabs(0, fab)
    A.regrid(0)
    assert len(A.levels) == 2
    A.set_level_fabs(1, fab)
    A.average_down_all()
    U0, m0 = A.valid(0)
    mass0 = U0[0][m0].sum()
    A.step(0.5)
    U, m = A.valid(0)
    assert abs(U[0][m].sum() - mass0) <= 1e-13 * mass0
    for l in range(2):
        V, mk = A.valid(l)
        s = V[5:][:, mk].sum(axis=0)
        assert np.allclose(s, V[0][mk], rtol=1e-14, atol=0)
