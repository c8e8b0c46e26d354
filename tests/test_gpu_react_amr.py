"""The reacting hierarchy on the GPU (ocfd_amr_create_reacting): species on
every subcycled level - chemistry over dt_l / 2 in 4 / 2^l substeps around the
RK2 multispecies flow step (Source/Advance.cpp:158-174,
Source/CHEM/FlowAdvance.cpp:9-90), flow and species flux registers and reflux,
renormalisation and average-down after the finer level's substeps
(Source/EBR.cpp:313-357) - against the CPU restatement (oracle/amr_oracle.py
with `react`) through a regrid, on a periodic H2/air box with a hot spot."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DX = 7.8125e-5     # the 128^3 / 1 cm reacting box's cell size
REACT = dict(dt=1e-8, chem_substeps=4, visc=True)


@pytest.fixture(scope="module")
def ctx():
    import ocfd
    return ocfd.Context()


def state_err(a, b):
    """grouped max-norm error of two 14-component states: density, energy and
    each partial density against their own maxima; momentum against rho * 800 m/s
    (the box starts at rest: momentum is a small residual)"""
    e = max(np.abs(a[0] - b[0]).max() / np.abs(b[0]).max(), np.abs(a[4] - b[4]).max() / np.abs(b[4]).max(),
            np.abs(a[1:4] - b[1:4]).max() / (800.0 * np.abs(b[0]).max()))
    for s in range(5, 14):
        e = max(e, float(np.abs(a[s] - b[s]).max() / max(np.abs(b[s]).max(), 1e-300)))
    return e


def make_pair(ctx, oracle, n0=(16, 16, 16), max_level=2, regrid_int=2, flux_fp32=False):
    from amr_oracle import AmrOracle
    from inputs import react_hot_spot_fab
    from ocfd.amr import Hierarchy
    from ocfd.level import chop_domain
    from test_gpu_amr import oracle_build
    fab = react_hot_spot_fab(oracle, n0, DX, radius_cells=3.0)
    kw = dict(max_level=max_level, blocking_factor=(4, 4, 4), max_grid_size=(8, 8, 8), n_error_buf=1,
              refine_dengrad=0.002)
    boxes0 = chop_domain(n0, (8, 8, 8))
    H = Hierarchy(ctx, boxes0, n0, (0, 0, 0), (0, 0, 0), (DX,) * 3, regrid_int=regrid_int,
                  react=dict(REACT, flux_fp32=flux_fp32), **kw)
    H.build(fab)
    A = AmrOracle(oracle, n0, (DX,) * 3, (0, 0, 0), (0, 0, 0), boxes0, react=REACT, **kw)
    oracle_build(A, fab)
    return H, A, fab


def compare(H, A, tol):
    assert H.all_grids() == A.grids()
    worst = 0.0
    for l in range(H.nlevels()):
        g, m = H.level_global(l)
        o, om = A.valid(l)
        assert (m == om).all()
        worst = max(worst, state_err(g[:, m], o[:, m]))
    assert worst <= tol, worst
    return worst


def test_reacting_hierarchy_matches_restatement(ctx, oracle):
    H, A, _ = make_pair(ctx, oracle)
    assert H.nlevels() == 3
    compare(H, A, 1e-15)
    for step in range(3):
        if step > 0 and step % 2 == 0:
            A.regrid(0)
        A.step(0.5)
        H.advance(1, 0.5)
        t, _ = H.time()
        assert abs(t - A.time) <= 1e-14 * A.time
        compare(H, A, 1e-9)
    # the chemistry ran on every level: OH forms in the hot spot
    for l in range(H.nlevels()):
        g, m = H.level_global(l)
        assert g[5 + 5][m].max() > 0.0
    H.close()


def test_reacting_hierarchy_conserves_mass_and_species_sum(ctx, oracle):
    """periodic box: total mass on level 0 (after average-down) conserved through
    the coarse steps with reflux; every level's partial densities sum to its
    density (renormalisation)"""
    H, _, _ = make_pair(ctx, oracle, regrid_int=0)
    g0, m0 = H.level_global(0)
    mass0 = g0[0][m0].sum()
    H.advance(3, 0.5)
    g, m = H.level_global(0)
    assert abs(g[0][m].sum() - mass0) <= 1e-12 * mass0
    for l in range(H.nlevels()):
        V, mk = H.level_global(l)
        assert np.allclose(V[5:][:, mk].sum(axis=0), V[0][mk], rtol=1e-13, atol=0)
    H.close()


def test_reacting_hierarchy_mixed_form_close(ctx, oracle):
    """the mixed form (FP32 split + WENO-Z of the flow and species faces) stays
    within 1e-6 of the FP64 form on every level after two coarse steps"""
    import ocfd
    Ha, _, _ = make_pair(ctx, oracle, regrid_int=0)
    Hb, _, _ = make_pair(ctx, oracle, regrid_int=0, flux_fp32=True)
    Ha.advance(2, 0.5)
    Hb.advance(2, 0.5, ocfd.FLUX_FP32)
    for l in range(Ha.nlevels()):
        a, m = Ha.level_global(l)
        b, _ = Hb.level_global(l)
        assert not np.array_equal(a[:, m], b[:, m])
        assert np.abs(a[0][m] - b[0][m]).sum() / np.abs(a[0][m]).sum() < 1e-6
    Ha.close()
    Hb.close()
