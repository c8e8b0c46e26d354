"""Cut-cell (EB) box RHS on the GPU against the oracle and the reference's
golden fixtures (tolerance 1e-12 norm-wise per conserved group)."""
import numpy as np
import pytest

import inputs
from conftest import golden

pytestmark = pytest.mark.gpu
TOL = 1e-12


def relerr(a, b):
    groups = [(0,), (1, 2, 3), (4,)]
    e = 0.0
    for g in groups:
        den = max(np.abs(b[list(g)]).max(), 1e-300)
        e = max(e, float(np.abs(a[list(g)] - b[list(g)]).max() / den))
    return e


@pytest.fixture(scope="module")
def ctx():
    import ocfd
    return ocfd.Context()


def to_dev(geom):
    import torch
    out = {}
    for k, v in geom.items():
        if k == "flag":
            out[k] = torch.from_numpy(np.ascontiguousarray(v).view(np.int32)).cuda()
        elif k in ("vfrac", "apx", "apy", "apz"):
            out[k] = torch.from_numpy(np.ascontiguousarray(v)).cuda()
    return out


def run_eb(ctx, S, geom, lo, dxinv, flags):
    import torch
    _, gz, gy, gx = S.shape
    nx, ny, nz = gx - 8, gy - 8, gz - 8
    hi = (lo[0] + nx - 1, lo[1] + ny - 1, lo[2] + nz - 1)
    dS = torch.full((5, nz, ny, nx), float("nan"), dtype=torch.float64, device="cuda")
    fl = [torch.full((5, nz + (d == 2), ny + (d == 1), nx + (d == 0)), float("nan"),
                     dtype=torch.float64, device="cuda") for d in range(3)]
    ctx.rhs_eb_box(torch.from_numpy(S).cuda(), dS, to_dev(geom), lo, hi, dxinv, flags, flux=fl)
    torch.cuda.synchronize()
    return dS.cpu().numpy(), [f.cpu().numpy() for f in fl]


@pytest.mark.parametrize("visc,red", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_eb_vs_golden(ctx, visc, red):
    g = golden(f"eb_v{visc}_r{red}")
    geom = {k: g[k] for k in ("flag", "vfrac", "apx", "apy", "apz")}
    dS, f = run_eb(ctx, np.ascontiguousarray(g["S"]), geom, (0, 0, 0), g["dxinv"], visc + 2 * red)
    assert relerr(dS, g["dSdt"]) < TOL
    for d, k in enumerate(("fx", "fy", "fz")):
        assert relerr(f[d], g[k]) < TOL


@pytest.mark.parametrize("shape,lo,seed", [((24, 20, 6), (40, -16, 3), 31), ((17, 33, 5), (0, 0, 0), 32)])
@pytest.mark.parametrize("visc", [0, 1])
def test_eb_vs_oracle(ctx, oracle, shape, lo, seed, visc):
    S = inputs.ideal_state(*shape, seed)
    geom = inputs.cylinder_box(*shape)
    for red in (0, 1):
        ref, rf = oracle.rhs_eb(S, geom, [5.0, 5.0, 5.0], visc, red)
        dS, f = run_eb(ctx, S, geom, lo, [5.0, 5.0, 5.0], visc + 2 * red)
        assert np.isfinite(dS).all()
        assert relerr(dS, ref) < TOL
        for d in range(3):
            assert relerr(f[d], rf[d]) < TOL
