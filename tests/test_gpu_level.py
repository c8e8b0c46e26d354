"""Level driver on the GPU: device ghost fill + fused SSP-RK3 steps + device CFL
dt, against the oracle's single-box RK3 (Shu-Osher form) on the same inputs,
and box-decomposition invariance (any box split gives bit-identical results)."""
import numpy as np
import pytest

from oracle import BCStruct
import inputs

pytestmark = pytest.mark.gpu


def oracle_bc(case):
    bc = BCStruct()
    bc.lo_bc[:] = list(case["lo_bc"]); bc.hi_bc[:] = list(case["hi_bc"])
    bc.dirichlet_case = case["bc_case"]
    bc.prob_lo[:] = list(case["prob_lo"]); bc.dx[:] = list(case["dx"])
    bc.dom_lo[:] = [0, 0, 0]
    bc.dom_hi[:] = [n - 1 for n in case["n"]]
    if case["bc_case"] == 1:
        bc.dmr_left[:] = list(case["case_params"][:5]); bc.dmr_right[:] = list(case["case_params"][5:10])
    return bc


def make_level(ctx, case, max_grid, tile=-1):
    from ocfd.level import Level, chop_domain
    n = case["n"]
    boxes = chop_domain(n, max_grid)
    return Level(ctx, boxes, tuple(x - 1 for x in n), case["lo_bc"], case["hi_bc"], case["dx"],
                 case["prob_lo"], case["bc_case"], case["case_params"], tile=tile)


def valid(G):
    return G[:, 4:-4, 4:-4, 4:-4]


def relerr(a, b):
    """max |a-b| / max |b| per conserved group: density, momentum vector, energy
    (a momentum component that is identically ~0 is measured against the
    momentum magnitude, not against its own rounding noise)."""
    groups = [(0,), (1, 2, 3), (4,)] + [(c,) for c in range(5, a.shape[0])]
    err = 0.0
    for g in groups:
        den = max(np.abs(b[list(g)]).max(), 1e-300)
        err = max(err, float(np.abs(a[list(g)] - b[list(g)]).max() / den))
    return err


@pytest.fixture(scope="module")
def ctx():
    import ocfd
    return ocfd.Context()


def run_gpu(ctx, case, nsteps, cfl, max_grid, flags=0, tile=-1):
    lev = make_level(ctx, case, max_grid, tile)
    lev.set_global(case["G"])
    lev.advance(nsteps, cfl, flags)
    t, dt = lev.time()
    out = lev.get_global()
    lev.close()
    return out, t


def run_oracle(oracle, case, nsteps, cfl, visc=False, gravity=False):
    S = np.ascontiguousarray(case["G"].copy())
    t, dts = oracle.advance_rk3(oracle_bc(case), S, cfl, nsteps, form=1, do_visc=visc, do_gravity=gravity)
    return valid(S), t


def test_sod_vs_oracle(ctx, oracle):
    from ocfd.cases import sod
    case = sod(64, 16, 4)
    ref, tr = run_oracle(oracle, case, 12, 0.5)
    got, tg = run_gpu(ctx, case, 12, 0.5, (64, 16, 4))
    assert tg == pytest.approx(tr, rel=1e-13)
    assert relerr(got, ref) < 1e-10


def test_first_dt_is_the_oracles(ctx, oracle):
    """The time step from the initial state, over boxes of several blocks, is the
    oracle's estdt bit for bit (the GPU reduces the largest signal speeds and
    divides once per block; correctly rounded division is monotone)."""
    from ocfd.cases import dmr, sod
    for case, grid in ((sod(64, 16, 4), (16, 8, 4)), (dmr(64, 16, 2), (24, 5, 2))):
        _, tr = run_oracle(oracle, case, 1, 0.5)
        _, tg = run_gpu(ctx, case, 1, 0.5, grid)
        assert tg == tr


def test_box_split_is_bit_identical(ctx):
    from ocfd.cases import sod
    case = sod(64, 16, 4)
    a, _ = run_gpu(ctx, case, 6, 0.5, (64, 16, 4))
    b, _ = run_gpu(ctx, case, 6, 0.5, (16, 8, 4))
    c, _ = run_gpu(ctx, case, 6, 0.5, (24, 5, 3))
    assert np.array_equal(a, b) and np.array_equal(a, c)


def test_tile_choice_is_bit_identical(ctx):
    from ocfd.cases import sod
    case = sod(48, 24, 8)
    ref, _ = run_gpu(ctx, case, 4, 0.5, (48, 24, 8), tile=0)
    for t in range(1, 6):
        got, _ = run_gpu(ctx, case, 4, 0.5, (48, 24, 8), tile=t)
        assert np.array_equal(got, ref), t


def test_dmr_vs_oracle(ctx, oracle):
    from ocfd.cases import dmr
    case = dmr(64, 16, 2)
    ref, tr = run_oracle(oracle, case, 10, 0.5)
    got, tg = run_gpu(ctx, case, 10, 0.5, (32, 8, 2))
    assert tg == pytest.approx(tr, rel=1e-13)
    assert relerr(got, ref) < 1e-10


def test_periodic_vs_oracle(ctx, oracle):
    n = (24, 16, 8)
    G = inputs.ideal_state(*n, seed=21, jump=False, mach=0.5)
    case = dict(G=G, n=n, dx=(1 / 24, 1 / 24, 1 / 24), prob_lo=(0, 0, 0), lo_bc=(0, 0, 0),
                hi_bc=(0, 0, 0), bc_case=0, case_params=())
    ref, tr = run_oracle(oracle, case, 8, 0.4)
    got, tg = run_gpu(ctx, case, 8, 0.4, (8, 8, 8))
    assert relerr(got, ref) < 1e-10


def test_viscous_level_vs_oracle(ctx, oracle):
    from ocfd.cases import sod
    case = sod(48, 12, 4)
    G = case["G"].copy()
    # dimensional air at ~300 K so that the viscous flux is visible
    G[0] *= 1.2; G[4] *= 1.0e5
    case = dict(case, G=G, dx=(1e-4, 1e-4, 1e-4), lo_bc=(2, 5, 4), hi_bc=(2, 5, 4))
    ref, tr = run_oracle(oracle, case, 6, 0.4, visc=True)
    got, tg = run_gpu(ctx, case, 6, 0.4, (16, 12, 4), flags=1)
    assert relerr(got, ref) < 1e-10


@pytest.mark.parametrize("scheme,order", [("RK2", 2), ("Euler", 1)])
def test_time_integration_vs_oracle(ctx, oracle, scheme, order):
    """ebr.time_integration = RK2 (the reference's default, Heun) and Euler
    (Source/Advance.cpp:115-138) on the DMR boundary functor over eight boxes,
    against the oracle's restatement in the reference's LinComb / Saxpy order"""
    from ocfd.cases import dmr
    case = dmr(64, 16, 2)
    S = np.ascontiguousarray(case["G"].copy())
    tr, _ = oracle.advance_rk(oracle_bc(case), S, 0.4, 8, order)
    lev = make_level(ctx, case, (16, 8, 2))
    lev.set_time_integration(scheme)
    lev.set_global(case["G"])
    lev.advance(8, 0.4)
    tg, _ = lev.time()
    got = lev.get_global()
    lev.close()
    assert tg == pytest.approx(tr, rel=1e-13)
    assert relerr(got, valid(S)) < 1e-10


def test_time_integration_switch_back_is_bit_identical(ctx):
    """RK2 then back to RK3 on the same level rebuilds the RK3 stage tables: the
    steps equal a level that never left RK3, bit for bit"""
    from ocfd.cases import sod
    case = sod(48, 16, 4)
    ref, _ = run_gpu(ctx, case, 5, 0.5, (16, 16, 4))
    lev = make_level(ctx, case, (16, 16, 4))
    lev.set_time_integration("RK2")
    lev.set_time_integration(3)
    lev.set_global(case["G"])
    lev.advance(5, 0.5)
    got = lev.get_global()
    lev.close()
    assert np.array_equal(got, ref)


def test_valid_copies(ctx):
    """copy_valid_out lists the valid cells box after box, (5, nz, ny, nx) each;
    a level whose ghost cells hold garbage and whose valid cells come from
    copy_valid_in (host or device buffer) steps bit-identically to one loaded
    with its ghost-filled FABs: every step fills the ghosts it reads"""
    import torch
    from ocfd.cases import dmr
    case = dmr(64, 16, 2)
    ref, _ = run_gpu(ctx, case, 4, 0.5, (16, 8, 2))
    G = case["G"]
    lev = make_level(ctx, case, (16, 8, 2))
    lev.set_global(G)
    v = lev.copy_valid_out()
    off = 0
    for lo, hi in lev.boxes:
        n = [hi[d] - lo[d] + 1 for d in range(3)]
        blk = v[off:off + 5 * n[0] * n[1] * n[2]].reshape(5, n[2], n[1], n[0])
        want = G[:, 4 + lo[2]:5 + hi[2], 4 + lo[1]:5 + hi[1], 4 + lo[0]:5 + hi[0]]
        assert np.array_equal(blk, want)
        off += blk.size
    assert off == v.size == lev.valid_elems()
    for src in (v, torch.from_numpy(v).cuda()):
        lev.copy_in(np.full(lev.elems, 1.0e30))
        lev.copy_valid_in(src)
        lev.advance(4, 0.5)
        assert np.array_equal(lev.get_global(), ref)
    dv = torch.empty(v.size, dtype=torch.float64, device="cuda")
    lev.copy_valid_out(dv)
    assert np.array_equal(dv.cpu().numpy(), lev.copy_valid_out())
    lev.close()


def test_gravity_level_vs_oracle(ctx, oracle):
    """A level advanced with OCFD_GRAVITY (the source in the fused stage of every
    regular box) against the oracle's RK3 with do_gravity; and the flag changes
    the result"""
    import ocfd
    from ocfd.cases import sod
    case = sod(48, 12, 8)
    G = case["G"].copy()
    G[0] *= 1.2; G[4] *= 1.0e5
    case = dict(case, G=G, dx=(1e-2, 1e-2, 1e-2))
    ref, tr = run_oracle(oracle, case, 6, 0.4, gravity=True)
    got, tg = run_gpu(ctx, case, 6, 0.4, (16, 12, 8), flags=ocfd.GRAVITY)
    nog, _ = run_gpu(ctx, case, 6, 0.4, (16, 12, 8))
    assert tg == pytest.approx(tr, rel=1e-13)
    assert relerr(got, ref) < 1e-10
    assert np.abs(got[3] - nog[3]).max() > 0
