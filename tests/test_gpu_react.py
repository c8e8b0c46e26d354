"""Reacting level on the GPU (ocfd_react_*): Strang-split Li-Dryer chemistry
around an RK2 / SSP-RK3 multispecies flow step and species renormalisation,
against the same sequence assembled from the oracle's box routines; batched
temperature-binned chemistry identical to the per-box form; the GPU state
constructor against the oracle's CKXTY / CKRHOY / CKUBMS."""
import numpy as np
import pytest

from oracle import BCStruct
from test_gpu_level import relerr

pytestmark = pytest.mark.gpu

NG = 4


@pytest.fixture(scope="module")
def ctx():
    import ocfd
    return ocfd.Context()


def small_case(ctx, n=16):
    from ocfd.cases import react_cube
    # a hot spot per box-sized region at n = 16, dx = 78 um as at 128^3 / 1 cm
    return react_cube(ctx, n=n, length=0.01 * n / 128, seed=7)


def oracle_step(orc, S, sp, dx, dt, rk, nsub, visc=True):
    """One step of the reference sequence on the whole periodic box (one box)."""
    n = S.shape[1] - 2 * NG
    bc = BCStruct()
    bc.lo_bc[:] = [0, 0, 0]
    bc.hi_bc[:] = [0, 0, 0]
    bc.dx[:] = list(dx)
    bc.dom_hi[:] = [n - 1] * 3
    inner = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))

    def chem_half(S, sp):
        for _ in range(nsub):
            a = np.ascontiguousarray(S[inner].reshape(5, -1))
            b = np.ascontiguousarray(sp[inner].reshape(9, -1))
            orc.chem_advance(a, b, 0.5 * dt / nsub)
            S[inner] = a.reshape(S[inner].shape)
            sp[inner] = b.reshape(sp[inner].shape)

    def L(S, sp):
        orc.fill_ghosts(bc, S)
        orc.fill_ghosts(bc, sp)
        dS, dSs, *_ = orc.rhs_chem(S, sp, tuple(1.0 / x for x in dx), do_visc=visc)
        return dS, dSs

    chem_half(S, sp)
    U0, V0 = S.copy(), sp.copy()
    if rk == 2:
        coef = [(0.0, 1.0), (0.5, 0.5)]
    else:
        coef = [(0.0, 1.0), (0.75, 0.25), (1.0 / 3.0, 2.0 / 3.0)]
    Us, Vs = S, sp
    for a, b in coef:
        dS, dSs = L(Us, Vs)
        Un, Vn = Us.copy(), Vs.copy()
        Un[inner] = a * U0[inner] + b * (Us[inner] + dt * dS)
        Vn[inner] = a * V0[inner] + b * (Vs[inner] + dt * dSs)
        Us, Vs = Un, Vn
    S[...] = Us
    sp[...] = Vs
    chem_half(S, sp)
    a = np.ascontiguousarray(S[inner].reshape(5, -1))
    b = np.ascontiguousarray(sp[inner].reshape(9, -1))
    orc.spec_renorm(a, b)
    sp[inner] = b.reshape(sp[inner].shape)


def run_gpu(ctx, case, boxes, steps, rk, binned=False, nsub=4, dt=1e-8, flux_fp32=False):
    from ocfd.react import Reactor
    n = case["n"]
    R = Reactor(ctx, boxes, tuple(x - 1 for x in n), case["dx"], dt=dt, rk_order=rk, chem_substeps=nsub,
                binned=binned, flux_fp32=flux_fp32)
    R.level.set_global(case["G"])
    R.advance(steps)
    out = R.level.get_global()
    R.close()
    return out


@pytest.mark.parametrize("rk", [2, 3])
def test_react_steps_vs_oracle(ctx, oracle, rk):
    from ocfd.level import chop_domain
    case = small_case(ctx)
    G = case["G"].copy()
    S = np.ascontiguousarray(G[:5])
    sp = np.ascontiguousarray(G[5:])
    steps = 2
    for _ in range(steps):
        oracle_step(oracle, S, sp, case["dx"], 1e-8, rk, 4)
    want = np.concatenate([S, sp])[:, NG:-NG, NG:-NG, NG:-NG]
    got = run_gpu(ctx, case, chop_domain(case["n"], 8), steps, rk)
    err = relerr(got, want)
    assert err < 1e-9, err
    # the chemistry did something: water forms in the hot spots
    assert want[5 + 2].max() > 0


def test_binned_chemistry_identical(ctx):
    from ocfd.level import chop_domain
    case = small_case(ctx)
    boxes = chop_domain(case["n"], 8)
    a = run_gpu(ctx, case, boxes, 2, 2, binned=False)
    b = run_gpu(ctx, case, boxes, 2, 2, binned=True)
    assert np.array_equal(a, b)


def test_state_tpx_vs_oracle(ctx, oracle):
    from ocfd.react import state_tpx
    rng = np.random.default_rng(3)
    T = rng.uniform(300.0, 2500.0, 50)
    p = rng.uniform(5e4, 5e5, 50)
    X = rng.random((9, 50))
    X /= X.sum(axis=0)
    G = state_tpx(ctx, T, p, X)
    for c in range(50):
        y = oracle.ckxty(X[:, c])
        rho = oracle.ckrhoy(p[c], T[c], y)
        r = rho * y
        assert G[0, c] == pytest.approx(rho, rel=1e-14)
        assert np.allclose(G[5:, c], r, rtol=1e-14, atol=0)
        assert G[4, c] == pytest.approx(oracle.ckubms(T[c], r), rel=1e-13)


def test_mixed_precision_flux_close_to_fp64(ctx):
    """The mixed form of the reacting level (FP32 split + WENO-Z of the flow and
    species face fluxes) stays within 1e-5 L1 of the FP64 form in density,
    pressure-bearing energy and Y_OH after a few steps, and is not identical to
    it (the FP32 path ran)."""
    from ocfd.level import chop_domain
    case = small_case(ctx, n=32)
    boxes = chop_domain(case["n"], 16)
    a = run_gpu(ctx, case, boxes, 4, 2)
    b = run_gpu(ctx, case, boxes, 4, 2, flux_fp32=True)
    assert np.isfinite(b).all() and not np.array_equal(a, b)
    l1 = lambda x, y: float(np.abs(x - y).sum() / np.abs(y).sum())
    assert l1(b[0], a[0]) < 1e-5 and l1(b[4], a[4]) < 1e-5
    assert l1(b[5 + 5] / b[0], a[5 + 5] / a[0]) < 1e-4


def _gsl(lo, hi, g):
    """slice of a grown global array (offset NG) over box lo..hi grown by g"""
    return (slice(None),) + tuple(slice(lo[d] + NG - g, hi[d] + NG + g + 1) for d in (2, 1, 0))


def oracle_step_eb(orc, S, sp, dx, dt, rk, nsub, geom, boxes, cls, visc=True):
    """One step of the reference sequence with an embedded body: per stage the
    box loop of compute_dSdt_multi (Source/CHEM/FlowAdvance.cpp:92-496: covered
    boxes dSdt = 0, regular boxes the multispecies chain, cut boxes the cut-cell
    chain), the chemistry on the boxes that are not covered
    (Source/CHEM/ChemAdvance.cpp:20), the species renormalisation everywhere."""
    from amr_oracle import BOX_COVERED, BOX_REGULAR
    nz, ny, nx = (m - 2 * NG for m in S.shape[1:])
    bc = BCStruct()
    bc.lo_bc[:] = [0, 0, 0]
    bc.hi_bc[:] = [0, 0, 0]
    bc.dx[:] = list(dx)
    bc.dom_hi[:] = [nx - 1, ny - 1, nz - 1]
    inner = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))
    dxinv = tuple(1.0 / x for x in dx)

    def chem_half(S, sp):
        for _ in range(nsub):
            for b, (lo, hi) in enumerate(boxes):
                if cls[b] == BOX_COVERED:
                    continue
                sl = _gsl(lo, hi, 0)
                a = np.ascontiguousarray(S[sl].reshape(5, -1))
                c = np.ascontiguousarray(sp[sl].reshape(9, -1))
                orc.chem_advance(a, c, 0.5 * dt / nsub)
                S[sl] = a.reshape(S[sl].shape)
                sp[sl] = c.reshape(sp[sl].shape)

    def L(S, sp):
        orc.fill_ghosts(bc, S)
        orc.fill_ghosts(bc, sp)
        dS = np.zeros((5, nz, ny, nx))
        dSs = np.zeros((9, nz, ny, nx))
        for b, (lo, hi) in enumerate(boxes):
            if cls[b] == BOX_COVERED:
                continue
            vs = (slice(None),) + tuple(slice(lo[d], hi[d] + 1) for d in (2, 1, 0))
            Sb = np.ascontiguousarray(S[_gsl(lo, hi, NG)])
            spb = np.ascontiguousarray(sp[_gsl(lo, hi, NG)])
            if cls[b] == BOX_REGULAR:
                d_, ds_, *_ = orc.rhs_chem(Sb, spb, dxinv, do_visc=visc)
            else:
                gb = {k: np.ascontiguousarray(geom[k][_gsl(lo, hi, NG)]) for k in ("flag", "vfrac")}
                for d, key in enumerate(("apx", "apy", "apz")):
                    h = list(hi)
                    h[d] += 1
                    gb[key] = np.ascontiguousarray(geom[key][(slice(None),) +
                                                             tuple(slice(lo[e], h[e] + 1) for e in (2, 1, 0))])
                d_, ds_, *_ = orc.rhs_chem(Sb, spb, dxinv, do_visc=visc, geom=gb)
            dS[vs] = d_
            dSs[vs] = ds_
        return dS, dSs

    chem_half(S, sp)
    U0, V0 = S.copy(), sp.copy()
    coef = [(0.0, 1.0), (0.5, 0.5)] if rk == 2 else [(0.0, 1.0), (0.75, 0.25), (1.0 / 3.0, 2.0 / 3.0)]
    Us, Vs = S, sp
    for a, b in coef:
        dS, dSs = L(Us, Vs)
        Un, Vn = Us.copy(), Vs.copy()
        Un[inner] = a * U0[inner] + b * (Us[inner] + dt * dS)
        Vn[inner] = a * V0[inner] + b * (Vs[inner] + dt * dSs)
        Us, Vs = Un, Vn
    S[...] = Us
    sp[...] = Vs
    chem_half(S, sp)
    a = np.ascontiguousarray(S[inner].reshape(5, -1))
    b = np.ascontiguousarray(sp[inner].reshape(9, -1))
    orc.spec_renorm(a, b)
    sp[inner] = b.reshape(sp[inner].shape)


@pytest.mark.parametrize("binned", [False, True])
def test_react_with_body_vs_oracle(ctx, oracle, binned):
    """A cylinder through the reacting box (48 x 48 x 8 cells, 8^3 boxes:
    covered, cut and regular boxes), RK2 and two steps against the box loop of
    the reference sequence; the per-box and binned chemistry agree"""
    from amr_oracle import box_classes
    from ocfd import geometry
    from ocfd.cases import react_cube
    from ocfd.level import chop_domain, eb_desc
    from ocfd.react import Reactor
    case = react_cube(ctx, n=48, length=0.01 * 48 / 128, seed=7)
    G = np.ascontiguousarray(case["G"][:, :8 + 2 * NG])
    n, dx = (48, 48, 8), case["dx"]
    centre, radius = (24 * dx[0], 24 * dx[1]), 12 * dx[0]
    geom = geometry.box_geometry(geometry.cylinder_phi(centre[0], centre[1], radius), (0, 0, 0), n, dx)
    boxes = chop_domain(n, 8)
    cls = box_classes(geom, boxes)
    assert {0, 1, 2} <= set(cls)
    S = np.ascontiguousarray(G[:5].copy())
    sp = np.ascontiguousarray(G[5:].copy())
    for _ in range(2):
        oracle_step_eb(oracle, S, sp, dx, 1e-8, 2, 4, geom, boxes, cls)
    want = np.concatenate([S, sp])[:, NG:-NG, NG:-NG, NG:-NG]
    R = Reactor(ctx, boxes, tuple(x - 1 for x in n), dx, dt=1e-8, rk_order=2, chem_substeps=4, binned=binned)
    R.set_eb(eb_desc(center=centre, radius=radius))
    assert R.box_classes() == cls
    R.level.set_global(G)
    R.advance(2)
    got = R.level.get_global()
    R.close()
    assert np.isfinite(got).all()
    err = relerr(got, want)
    assert err < 1e-9, err
