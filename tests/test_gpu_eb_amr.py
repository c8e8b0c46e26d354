"""AMR hierarchy cut by an embedded cylinder (ocfd_amr_set_eb) on the GPU:
the Mach 2 jet past a cylinder at a small size, checked against the CPU
restatement with the body (oracle/amr_oracle.py): box classes on every level,
hierarchy construction (volume-fraction average-down, piecewise-constant
interpolation next to the body) and coarse steps with regridding (cut-cell
scheme, area-weighted flux registers, reflux divided by volume fractions)."""
import numpy as np
import pytest

from test_gpu_amr import compare_levels, make_hierarchy, oracle_build

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import ocfd
    return ocfd.Context()


def small_jet(max_grid0=16):
    from ocfd.cases import jet_eb_amr
    from ocfd.level import chop_domain
    case = jet_eb_amr(nx=64, ny=32, nz=4, max_level=2, blocking_factor=8, max_grid=16, n_error_buf=1,
                      refine_dengrad=0.1, regrid_int=2)
    case["boxes0"] = chop_domain(case["n"], max_grid0)
    return case


def make_pair(ctx, oracle, case, time_integration=3):
    from amr_oracle import AmrOracle
    from ocfd.level import eb_desc
    H = make_hierarchy(ctx, case)
    H.set_time_integration(time_integration)
    H.set_eb(eb_desc(center=case["eb"]["center"], radius=case["eb"]["radius"],
                     redistribute=case["eb"]["redistribute"]))
    H.build(case["fab"])
    A = AmrOracle(oracle, case["n"], case["dx"], case["lo_bc"], case["hi_bc"], case["boxes0"], case["prob_lo"],
                  case["bc_case"], case["case_params"], case["max_level"], case["blocking_factor"],
                  case["max_grid_size"], case["n_error_buf"], case["refine_dengrad"], eb=case["eb"],
                  time_integration=time_integration)
    oracle_build(A, case["fab"])
    return H, A


def test_jet_eb_build_matches_oracle(ctx, oracle):
    case = small_jet()
    H, A = make_pair(ctx, oracle, case)
    assert H.nlevels() == 3
    for l in range(H.nlevels()):
        assert H.box_classes(l) == A.classes(l), l
    # the body cuts boxes of the base level
    assert 1 in H.box_classes(0)
    compare_levels(H, A, 1e-15)


@pytest.mark.parametrize("order", [3, 2])
def test_jet_eb_steps_match_oracle(ctx, oracle, order):
    """SSP-RK3, and RK2 (the time integration of the reference's jet inputs)"""
    case = small_jet()
    H, A = make_pair(ctx, oracle, case, time_integration=order)
    cfl = 0.5
    for step in range(4):
        if step > 0 and step % case["regrid_int"] == 0:
            A.regrid(0)
        A.step(cfl)
        H.advance(1, cfl)
        t, _ = H.time()
        assert abs(t - A.time) <= 1e-13 * A.time
        for l in range(H.nlevels()):
            assert H.box_classes(l) == A.classes(l)
        compare_levels(H, A, 1e-11)
        g, m = H.level_global(0)
        assert 0.0 < g[0][m].min() and g[0][m].max() < 10.0
    for l in range(H.nlevels()):
        g, m = H.level_global(l)
        # bounded: the jet's density lies between 1.0 and 1.4, the bow shock
        # compresses it a few times, the wake expands it
        assert np.isfinite(g[:, m]).all() and 0.0 < g[0][m].min() and g[0][m].max() < 10.0


def test_jet_eb_forms_and_schedules(ctx):
    """On the cut hierarchy: the autotuned schedules give the same state as the
    default ones bit for bit, the reference's per-box execution model too, and
    the mixed form stays within 1e-6 L1 of the FP64 form in density and energy
    after coarse steps on identical grids."""
    import ocfd
    from ocfd.level import eb_desc
    case = small_jet()

    def run(flags, tune=False, steps=3):
        H = make_hierarchy(ctx, case, regrid_int=0)
        H.set_eb(eb_desc(center=case["eb"]["center"], radius=case["eb"]["radius"],
                         redistribute=case["eb"]["redistribute"]))
        H.build(case["fab"])
        if tune:
            H.autotune(flags & ocfd.FLUX_FP32, reps=2)
        H.advance(steps, 0.5, flags)
        out = [H.level_global(l) for l in range(H.nlevels())]
        H.close()
        return out

    base = run(0)
    for other in (run(0, tune=True), run(ocfd.PER_BOX)):
        for (a, m), (b, _) in zip(base, other):
            assert np.array_equal(a[:, m], b[:, m])
    mixed = run(ocfd.FLUX_FP32)
    l1 = lambda x, y: float(np.abs(x - y).sum() / np.abs(y).sum())
    for (a, m), (b, _) in zip(base, mixed):
        assert not np.array_equal(a[:, m], b[:, m])
        assert l1(b[0][m], a[0][m]) < 1e-6 and l1(b[4][m], a[4][m]) < 1e-6
