"""Multispecies box RHS on the GPU against the oracle and the reference's golden
fixture.  Flow and species groups are compared norm-wise at 1e-11 (the real-gas
temperature and transport use exp/log/pow, so a few ulps differ from the host)."""
import numpy as np
import pytest

import inputs
from conftest import golden

pytestmark = pytest.mark.gpu
TOL = 1e-11


def grel(a, b, groups):
    e = 0.0
    for g in groups:
        den = max(np.abs(b[list(g)]).max(), 1e-300)
        e = max(e, float(np.abs(a[list(g)] - b[list(g)]).max() / den))
    return e


FLOW = [(0,), (1, 2, 3), (4,)]
SPEC = [tuple(range(9))]


@pytest.fixture(scope="module")
def ctx():
    import ocfd
    return ocfd.Context()


def run_chem_rhs(ctx, S, sp, lo, dxinv, visc, geom=None):
    import torch
    _, gz, gy, gx = S.shape
    nx, ny, nz = gx - 8, gy - 8, gz - 8
    hi = (lo[0] + nx - 1, lo[1] + ny - 1, lo[2] + nz - 1)
    d = lambda *s: torch.full(s, float("nan"), dtype=torch.float64, device="cuda")
    dS, dSs = d(5, nz, ny, nx), d(9, nz, ny, nx)
    fl = [d(5, nz + (k == 2), ny + (k == 1), nx + (k == 0)) for k in range(3)]
    fs = [d(9, nz + (k == 2), ny + (k == 1), nx + (k == 0)) for k in range(3)]
    St = torch.from_numpy(np.ascontiguousarray(S)).cuda()
    Rt = torch.from_numpy(np.ascontiguousarray(sp)).cuda()
    if geom is None:
        ctx.rhs_chem_box(St, Rt, dS, dSs, lo, hi, dxinv, int(visc), flux=fl, flux_spec=fs)
    else:
        from test_gpu_eb import to_dev
        ctx.rhs_chem_eb_box(St, Rt, dS, dSs, to_dev(geom), lo, hi, dxinv, int(visc), flux=fl, flux_spec=fs)
    torch.cuda.synchronize()
    return (dS.cpu().numpy(), dSs.cpu().numpy(), [x.cpu().numpy() for x in fl], [x.cpu().numpy() for x in fs])


def test_chem_rhs_vs_golden(ctx):
    g = golden("chem_regular")
    dS, dSs, f, fs = run_chem_rhs(ctx, g["S"], g["spec"], (0, 0, 0), g["dxinv"], True)
    assert grel(dS, g["dSdt"], FLOW) < TOL
    assert grel(dSs, g["dSdt_spec"], SPEC) < TOL
    for d, k in enumerate(("fxs", "fys", "fzs")):
        assert grel(fs[d], g[k], SPEC) < TOL


@pytest.mark.parametrize("visc", [False, True])
@pytest.mark.parametrize("shape,lo", [((12, 10, 7), (0, 0, 0)), ((9, 16, 5), (-3, 20, 7))])
def test_chem_rhs_vs_oracle(ctx, oracle, visc, shape, lo):
    S, sp = inputs.chem_state(*shape, seed=91, oracle=oracle)
    dxinv = [1.0e4, 1.2e4, 0.8e4]
    ref = oracle.rhs_chem(S, sp, dxinv, do_visc=visc)
    got = run_chem_rhs(ctx, S, sp, lo, dxinv, visc)
    assert np.isfinite(got[0]).all() and np.isfinite(got[1]).all()
    assert grel(got[0], ref[0], FLOW) < TOL
    assert grel(got[1], ref[1], SPEC) < TOL
    for d in range(3):
        assert grel(got[2][d], ref[2][d], FLOW) < TOL
        assert grel(got[3][d], ref[3][d], SPEC) < TOL


def test_chem_eb_rhs_vs_golden(ctx):
    g = golden("chem_eb")
    geom = {k: g[k] for k in ("flag", "vfrac", "apx", "apy", "apz")}
    dS, dSs, f, fs = run_chem_rhs(ctx, g["S"], g["spec"], (0, 0, 0), g["dxinv"], True, geom=geom)
    assert np.array_equal(dS, g["dSdt"])     # zero, as in the reference
    assert grel(dSs, g["dSdt_spec"], SPEC) < TOL
    for d, k in enumerate(("fxs", "fys", "fzs")):
        assert grel(fs[d], g[k], SPEC) < TOL


@pytest.mark.parametrize("visc", [False, True])
def test_chem_eb_rhs_vs_oracle(ctx, oracle, visc):
    shape = (12, 11, 5)
    S, sp = inputs.chem_state(*shape, seed=93, oracle=oracle)
    geom = inputs.cylinder_box(*shape)
    dxinv = [1.0e4, 1.0e4, 1.0e4]
    ref = oracle.rhs_chem(S, sp, dxinv, do_visc=visc, geom=geom)
    got = run_chem_rhs(ctx, S, sp, (0, 0, 0), dxinv, visc, geom=geom)
    assert np.isfinite(got[1]).all()
    assert np.array_equal(got[0], ref[0])
    assert grel(got[1], ref[1], SPEC) < TOL
    for d in range(3):
        assert grel(got[2][d], ref[2][d], FLOW) < TOL
        assert grel(got[3][d], ref[3][d], SPEC) < TOL
