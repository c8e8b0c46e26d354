"""AMR hierarchy on the GPU (ocfd_amr_*): subcycled SSP-RK3 with time-interpolated
coarse-fine ghosts, reflux, average-down and density-gradient regridding,
checked against the CPU restatement (oracle/amr_oracle.py) and by the
properties the coarse-fine operators must have: conservation with reflux,
exactness of the interpolation on linear data, free-stream preservation,
invariance to the level-0 box decomposition."""
import numpy as np
import pytest

from test_gpu_level import relerr

pytestmark = pytest.mark.gpu

NG = 4


@pytest.fixture(scope="module")
def ctx():
    import ocfd
    return ocfd.Context()


def small_dmr(max_grid0=16):
    from ocfd.cases import dmr_amr
    from ocfd.level import chop_domain
    case = dmr_amr(nx=64, ny=16, nz=2, max_level=2, blocking_factor=8, max_grid=16, n_error_buf=1,
                   regrid_int=2)
    case["boxes0"] = chop_domain(case["n"], max_grid0)
    return case


def make_hierarchy(ctx, case, regrid_int=None):
    from ocfd.amr import Hierarchy
    return Hierarchy(ctx, case["boxes0"], case["n"], case["lo_bc"], case["hi_bc"], case["dx"],
                     case["prob_lo"], case["bc_case"], case["case_params"], case["max_level"],
                     case["blocking_factor"], case["max_grid_size"], case["n_error_buf"],
                     case["regrid_int"] if regrid_int is None else regrid_int, case["refine_dengrad"])


def make_oracle(orc, case, time_integration=3):
    from amr_oracle import AmrOracle
    return AmrOracle(orc, case["n"], case["dx"], case["lo_bc"], case["hi_bc"], case["boxes0"], case["prob_lo"],
                     case["bc_case"], case["case_params"], case["max_level"], case["blocking_factor"],
                     case["max_grid_size"], case["n_error_buf"], case["refine_dengrad"],
                     time_integration=time_integration)


def oracle_build(A, fab):
    A.set_level_fabs(0, fab)
    for lev in range(A.max_level):
        if len(A.levels) != lev + 1:
            break
        A.regrid(lev)
        if len(A.levels) == lev + 2:
            A.set_level_fabs(lev + 1, fab)
    A.average_down_all()


def compare_levels(H, A, tol):
    assert H.all_grids() == A.grids()
    worst = 0.0
    for l in range(H.nlevels()):
        g, m = H.level_global(l)
        o, om = A.valid(l)
        assert (m == om).all()
        worst = max(worst, relerr(g[:, m], o[:, m]))
    assert worst < tol, worst
    return worst


def test_dmr_build_matches_oracle(ctx, oracle):
    case = small_dmr()
    H = make_hierarchy(ctx, case)
    H.build(case["fab"])
    A = make_oracle(oracle, case)
    oracle_build(A, case["fab"])
    assert H.nlevels() == 3
    compare_levels(H, A, 1e-15)
    leaf, allc = H.cell_steps()
    assert 0 < leaf <= allc


def test_dmr_steps_match_oracle(ctx, oracle):
    """three coarse steps with a regrid before the third, every level within
    1e-11 (grouped relative max error) of the CPU restatement"""
    case = small_dmr()
    H = make_hierarchy(ctx, case)
    H.build(case["fab"])
    A = make_oracle(oracle, case)
    oracle_build(A, case["fab"])
    cfl = 0.5
    for step in range(3):
        if step > 0 and step % case["regrid_int"] == 0:
            A.regrid(0)
        A.step(cfl)
        H.advance(1, cfl)
        t, dt = H.time()
        assert abs(t - A.time) <= 1e-14 * A.time
        compare_levels(H, A, 1e-11)


def test_box_split_invariance(ctx):
    """the level-0 decomposition does not change any level's result"""
    outs = []
    for mg in (16, 32):
        case = small_dmr(max_grid0=mg)
        H = make_hierarchy(ctx, case)
        H.build(case["fab"])
        H.advance(3, 0.5)
        outs.append([H.level_global(l)[0] for l in range(H.nlevels())] + [H.all_grids()])
    a, b = outs
    assert a[-1][1:] == b[-1][1:]
    for x, y in zip(a[:-1], b[:-1]):
        assert np.array_equal(np.nan_to_num(x, nan=-7.0), np.nan_to_num(y, nan=-7.0))


def periodic_case(n=(32, 32, 8)):
    from ocfd.level import chop_domain
    dx = 1.0 / n[0]

    def fab(lev, lo, hi, d):
        x = (np.arange(lo[0] - NG, hi[0] + NG + 1) + 0.5) * d[0]
        y = (np.arange(lo[1] - NG, hi[1] + NG + 1) + 0.5) * d[1]
        z = (np.arange(lo[2] - NG, hi[2] + NG + 1) + 0.5) * d[2]
        Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
        r2 = (X - 0.5) ** 2 + (Y - 0.5) ** 2 + (Z - 0.125) ** 2
        rho = 1.0 + 0.5 * np.exp(-r2 / 0.02)
        u, v, w, p = 1.0, 0.5, 0.25, 1.0
        return np.stack([rho, rho * u, rho * v, rho * w, p / 0.4 + 0.5 * rho * (u * u + v * v + w * w)])
    return dict(n=n, dx=(dx, dx, dx), prob_lo=(0.0, 0.0, 0.0), lo_bc=(0, 0, 0), hi_bc=(0, 0, 0), bc_case=0,
                case_params=(), max_level=1, blocking_factor=(8, 8, 8), max_grid_size=(16, 16, 16),
                n_error_buf=1, refine_dengrad=0.05, regrid_int=0, fab=fab, boxes0=chop_domain(n, 16))


# two fine boxes of level 1 (domain 64 x 64 x 16); the second one touches the
# periodic boundary x = 63 | 0
PERIODIC_FINE = [((16, 16, 4), (39, 31, 11)), ((56, 40, 0), (63, 55, 15))]


@pytest.mark.parametrize("scheme,order", [("RK2", 2), ("Euler", 1)])
def test_dmr_steps_match_oracle_time_integration(ctx, oracle, scheme, order):
    """RK2 (Heun) and Euler on the subcycled hierarchy: coarse-fine ghosts by
    linear interpolation between the coarse old and new states (FillPatch), flux
    registers weighted 0.5 dt / dt, three coarse steps with a regrid"""
    case = small_dmr()
    H = make_hierarchy(ctx, case)
    H.set_time_integration(scheme)
    H.build(case["fab"])
    A = make_oracle(oracle, case, time_integration=order)
    oracle_build(A, case["fab"])
    cfl = 0.4
    for step in range(3):
        if step > 0 and step % case["regrid_int"] == 0:
            A.regrid(0)
        A.step(cfl)
        H.advance(1, cfl)
        t, _ = H.time()
        assert abs(t - A.time) <= 1e-14 * A.time
        compare_levels(H, A, 1e-11)


def test_valid_copies_step_like_fabs(ctx):
    """every level loaded through copy_valid_in over ghost cells holding garbage
    steps bit-identically (two coarse steps, a regrid) to the hierarchy restored
    from its ghost-filled FABs"""
    case = small_dmr()
    H = make_hierarchy(ctx, case)
    H.build(case["fab"])
    H.advance(1, 0.5)
    snap = H.snapshot()
    H.restore(snap)
    H.advance(2, 0.5)
    ref = [H.level_global(l) for l in range(H.nlevels())]
    grids = H.all_grids()
    H.restore(snap)
    valid = [H.copy_valid_out(l) for l in range(H.nlevels())]
    for l in range(H.nlevels()):
        H.copy_in(l, np.full(H.state_elems(l), 1.0e30))
        H.copy_valid_in(l, valid[l])
    H.advance(2, 0.5)
    assert H.all_grids() == grids
    for l in range(H.nlevels()):
        g, m = H.level_global(l)
        assert (m == ref[l][1]).all() and np.array_equal(g[:, m], ref[l][0][:, m]), l


def totals(H):
    g, m = H.level_global(0)
    return g[:, m].sum(axis=1)


def test_reflux_conserves_periodic(ctx, oracle):
    case = periodic_case()
    H = make_hierarchy(ctx, case)
    L0 = H.level(0)
    L0.copy_in(L0.pack_fabs(lambda lo, hi: case["fab"](0, lo, hi, case["dx"])))
    H.set_grids([PERIODIC_FINE])
    H.average_down()
    H.set_time(0.0)
    s0 = totals(H)
    H.advance(4, 0.5)
    s1 = totals(H)
    rel = np.abs(s1 - s0) / np.maximum(np.abs(s0), 1e-300)
    assert rel.max() < 1e-13, rel
    # the same steps on the CPU restatement
    from amr_oracle import AmrOracle
    A = AmrOracle(oracle, case["n"], case["dx"], case["lo_bc"], case["hi_bc"], case["boxes0"], max_level=1,
                  blocking_factor=(8, 8, 8), max_grid_size=(16, 16, 16))
    A.set_level_fabs(0, case["fab"])
    A.fill_all_sync()
    A.apply_grids(0, [PERIODIC_FINE])
    A.average_down_all()
    for _ in range(4):
        A.step(0.5)
    compare_levels(H, A, 1e-11)


def test_interpolation_exact_on_linear_data(ctx):
    """a new fine level and its coarse-fine ghost cells reproduce linear data"""
    from ocfd.level import chop_domain
    n = (32, 32, 16)
    dx = 1.0 / 32
    grad = np.array([[0.3, -0.2, 0.1], [1.0, 2.0, -3.0], [0.5, 0.25, 0.125], [-1.0, 1.0, 0.5], [4.0, -2.0, 1.0]])
    base = np.array([2.0, 0.1, -0.2, 0.3, 5.0])

    def fab(lo, hi, d):
        x = (np.arange(lo[0] - NG, hi[0] + NG + 1) + 0.5) * d[0]
        y = (np.arange(lo[1] - NG, hi[1] + NG + 1) + 0.5) * d[1]
        z = (np.arange(lo[2] - NG, hi[2] + NG + 1) + 0.5) * d[2]
        Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
        return np.stack([base[c] + grad[c, 0] * X + grad[c, 1] * Y + grad[c, 2] * Z for c in range(5)])
    case = dict(n=n, dx=(dx,) * 3, prob_lo=(0.0,) * 3, lo_bc=(2, 2, 2), hi_bc=(2, 2, 2), bc_case=0, case_params=(),
                max_level=1, blocking_factor=(8, 8, 8), max_grid_size=(16, 16, 16), n_error_buf=1,
                refine_dengrad=0.05, regrid_int=0, boxes0=chop_domain(n, 16))
    H = make_hierarchy(ctx, case)
    L0 = H.level(0)
    L0.copy_in(L0.pack_fabs(lambda lo, hi: fab(lo, hi, case["dx"])))
    fine = [((16, 16, 8), (31, 31, 23)), ((32, 16, 8), (47, 39, 23))]
    H.set_grids([fine])
    H.fill_ghosts()
    L1 = H.level(1)
    flat = L1.copy_out()
    off = 0
    fd = H.dx(1)
    for lo, hi in L1.boxes:
        shape = (5, hi[2] - lo[2] + 1 + 2 * NG, hi[1] - lo[1] + 1 + 2 * NG, hi[0] - lo[0] + 1 + 2 * NG)
        size = int(np.prod(shape))
        got = flat[off:off + size].reshape(shape)[:, 1:-1, 1:-1, 1:-1]   # the 3 filled ghost layers
        off += size
        want = fab(lo, hi, fd)[:, 1:-1, 1:-1, 1:-1]
        err = np.abs(got - want).max() / np.abs(want).max()
        assert err < 1e-14, (lo, hi, err)


def test_free_stream_three_levels(ctx):
    from ocfd.level import chop_domain
    n = (32, 16, 8)
    dx = 1.0 / 32
    state = np.array([1.3, 1.3 * 0.7, -1.3 * 0.4, 1.3 * 0.2, 2.0 / 0.4 + 0.5 * 1.3 * (0.49 + 0.16 + 0.04)])

    def fab(lev, lo, hi, d):
        shape = (hi[2] - lo[2] + 1 + 2 * NG, hi[1] - lo[1] + 1 + 2 * NG, hi[0] - lo[0] + 1 + 2 * NG)
        return np.stack([np.full(shape, s) for s in state])
    case = dict(n=n, dx=(dx,) * 3, prob_lo=(0.0,) * 3, lo_bc=(0, 0, 0), hi_bc=(0, 0, 0), bc_case=0, case_params=(),
                max_level=2, blocking_factor=(8, 8, 8), max_grid_size=(16, 16, 16), n_error_buf=1,
                refine_dengrad=0.05, regrid_int=0, boxes0=chop_domain(n, 16))
    H = make_hierarchy(ctx, case)
    L0 = H.level(0)
    L0.copy_in(L0.pack_fabs(lambda lo, hi: fab(0, lo, hi, case["dx"])))
    l1 = [((16, 8, 0), (47, 23, 15))]
    l2 = [((40, 24, 8), (71, 39, 23)), ((72, 24, 8), (87, 39, 23))]
    H.set_grids([l1, l2])
    H.set_time(0.0)
    H.advance(5, 0.5)
    assert H.nlevels() == 3
    for l in range(3):
        g, m = H.level_global(l)
        dev = np.abs(g[:, m] - state[:, None]).max(axis=1) / np.abs(state).max()
        assert dev.max() < 1e-13, (l, dev)


def test_mixed_form_close_on_hierarchy(ctx):
    """FP32 flux form on the same (frozen) grids stays within 1e-4 L1 of FP64"""
    import ocfd
    case = small_dmr()
    res = []
    for flags in (0, ocfd.FLUX_FP32):
        H = make_hierarchy(ctx, case, regrid_int=0)
        H.build(case["fab"])
        H.set_stop_time(0.01)
        H.advance(20, 0.5, flags)
        g, m = H.level_global(0)
        res.append((H.time()[0], g[:, m]))
    (t0, a), (t1, b) = res
    assert t0 == pytest.approx(0.01, abs=1e-15) and t1 == pytest.approx(0.01, abs=1e-15)
    l1 = np.abs(a[0] - b[0]).sum() / np.abs(a[0]).sum()
    assert l1 < 1e-4, l1


def test_plotfile_of_hierarchy(ctx, tmp_path):
    """the hierarchy's plotfile holds every level's valid state and the derived
    ux, uy, uz, pressure; fcompare of the FP32 and FP64 runs on the same grids
    gives the L1 norm computed from the device data"""
    import ocfd
    from ocfd import plotfile
    from test_plotfile import parse
    case = small_dmr()
    runs = {}
    for flags in (0, ocfd.FLUX_FP32):
        H = make_hierarchy(ctx, case, regrid_int=0)
        H.build(case["fab"])
        H.advance(3, 0.5, flags)
        p = str(tmp_path / ("plt_%d" % flags))
        plotfile.write_hierarchy(H, p, step=3)
        runs[flags] = (p, [H.level_global(l) for l in range(H.nlevels())], H.time()[0])
    p, glob, t = runs[0]
    d = parse(p)
    assert d["names"] == ["rho", "xmom", "ymom", "zmom", "Eden", "ux", "uy", "uz", "pressure"]
    assert d["finest"] == len(glob) - 1 and d["time"] == t and d["steps"] == [3, 6, 12][:len(glob)]
    for l, (g, m) in enumerate(glob):
        for lo, hi, arr in d["data"][l]:
            sl = (slice(None), slice(lo[2], hi[2] + 1), slice(lo[1], hi[1] + 1), slice(lo[0], hi[0] + 1))
            U = g[sl]
            assert np.array_equal(arr[:5], U)
            assert np.array_equal(arr[5], U[1] / U[0])
            pres = 0.4 * (U[4] - 0.5 / U[0] * (U[1] * U[1] + U[2] * U[2] + U[3] * U[3]))
            assert np.allclose(arr[8], pres, rtol=1e-15, atol=0)
    r = plotfile.compare(runs[0][0], runs[ocfd.FLUX_FP32][0], norm=1)
    for l, ((a, m), (b, _)) in enumerate(zip(runs[0][1], runs[ocfd.FLUX_FP32][1])):
        l1 = np.abs(b[0][m] - a[0][m]).sum() / np.abs(a[0][m]).sum()
        assert r["rel"][l, 0] == pytest.approx(l1, rel=1e-9)
        assert r["rel"][l, 0] < 1e-4
