"""Regular-box RHS on the GPU against the oracle (and the reference's golden
fixtures), through the C ABI.  Tolerance: max|gpu - ref| / max|ref| <= 1e-12 per
component (FMA contraction on the GPU is the only difference)."""
import numpy as np
import pytest

import inputs
from conftest import golden

pytestmark = pytest.mark.gpu
TOL = 1e-12


def relerr(a, b):
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / (den if den > 0 else 1.0))


@pytest.fixture(scope="module")
def ctx():
    import ocfd
    return ocfd.Context()


def run_gpu(ctx, S, lo, dxinv, flags=0, with_flux=True):
    import torch
    nc, gz, gy, gx = S.shape
    nx, ny, nz = gx - 8, gy - 8, gz - 8
    hi = (lo[0] + nx - 1, lo[1] + ny - 1, lo[2] + nz - 1)
    St = torch.from_numpy(S).cuda()
    dS = torch.full((5, nz, ny, nx), float("nan"), dtype=torch.float64, device="cuda")
    fl = None
    if with_flux:
        fl = [torch.full((5, nz + (d == 2), ny + (d == 1), nx + (d == 0)), float("nan"),
                         dtype=torch.float64, device="cuda") for d in range(3)]
    ctx.rhs_regular_box(St, dS, lo, hi, dxinv, flags, flux=fl)
    torch.cuda.synchronize()
    return dS.cpu().numpy(), [f.cpu().numpy() for f in fl] if fl else None


@pytest.mark.parametrize("name", ["regular_inviscid", "regular_viscous"])
def test_regular_vs_golden(ctx, name):
    g = golden(name)
    visc = name.endswith("viscous")
    dS, f = run_gpu(ctx, np.ascontiguousarray(g["S"]), (0, 0, 0), g["dxinv"], flags=int(visc))
    for n in range(5):
        assert relerr(dS[n], g["dSdt"][n]) < TOL, n
    for d, k in enumerate(("fx", "fy", "fz")):
        for n in range(5):
            assert relerr(f[d][n], g[k][n]) < TOL


@pytest.mark.parametrize("shape,lo,seed", [
    ((16, 16, 16), (0, 0, 0), 1),
    ((21, 13, 9), (32, -8, 5), 2),     # ragged: no tile shape divides it, non-zero origin
    ((64, 32, 4), (0, 0, 0), 3),       # thin slab
    ((33, 7, 2), (-4, 100, 0), 4),
    ((1, 1, 1), (5, 5, 5), 5),         # single cell
])
@pytest.mark.parametrize("visc", [False, True])
def test_regular_vs_oracle(ctx, oracle, shape, lo, seed, visc):
    S = inputs.ideal_state(*shape, seed)
    if visc:   # dimensional air-like state so the viscous terms matter
        S = S.copy(); S[0] *= 1.2; S[1:4] *= 360.0; S[4] *= 1.0e5
    dxinv = [1.0e4, 1.2e4, 0.9e4] if visc else [shape[0] * 1.0, 9.0, 7.0]
    ref, rf = oracle.rhs_regular(S, dxinv, do_visc=visc)
    dS, f = run_gpu(ctx, S, lo, dxinv, flags=int(visc))
    assert np.isfinite(dS).all()
    for n in range(5):
        assert relerr(dS[n], ref[n]) < TOL, (n, relerr(dS[n], ref[n]))
    for d in range(3):
        assert np.isfinite(f[d]).all()
        for n in range(5):
            assert relerr(f[d][n], rf[d][n]) < TOL


def test_regular_no_flux_output(ctx, oracle):
    S = inputs.ideal_state(24, 20, 12, 7)
    ref, _ = oracle.rhs_regular(S, [3.0, 3.0, 3.0])
    dS, _ = run_gpu(ctx, S, (0, 0, 0), [3.0, 3.0, 3.0], with_flux=False)
    assert relerr(dS, ref) < TOL


def test_regular_rejects_short_ghosts(ctx):
    import torch
    import ocfd
    S = torch.zeros((5, 10, 10, 10), dtype=torch.float64, device="cuda")
    dS = torch.zeros((5, 8, 8, 8), dtype=torch.float64, device="cuda")
    with pytest.raises(ocfd.OcfdError) as e:
        ctx.rhs_regular_box(S, dS, (0, 0, 0), (7, 7, 7), [1.0, 1.0, 1.0], S_begin=(-1, -1, -1))
    assert e.value.status == 1


def _periodic_grown(core, n):
    """(5, nz+8, ny+8, nx+8) state of box 0..n-1 (grown by 4) tiled from the
    8-periodic cell pattern core (5, 8, 8, 8): grown index g holds core[(g-4) % 8]."""
    reps = [(m + 12) // 8 + 1 for m in (n[2], n[1], n[0])]
    big = core.repeat(1, *reps)
    return big[:, 4:12 + n[2], 4:12 + n[1], 4:12 + n[0]].contiguous()


@pytest.mark.parametrize("flags", [0, 4])
def test_large_box_equals_periodic_tile(ctx, flags):
    """One box of 512 x 256 x 64 cells (8.4 M cells, thousands of tiles in one
    launch) holding an 8-periodic state: its RHS is the RHS of the 8^3 box with
    periodic ghosts, tiled, bit for bit in the FP64 and the mixed form (the
    arithmetic of a cell depends on neither the box nor the tile decomposition)"""
    import torch
    P = inputs.ideal_state(8, 8, 8, 11)
    core = torch.from_numpy(np.ascontiguousarray(P[:, 4:12, 4:12, 4:12])).cuda()
    dx = [8.0, 8.0, 8.0]
    Ss = _periodic_grown(core, (8, 8, 8))
    dSs = torch.empty((5, 8, 8, 8), dtype=torch.float64, device="cuda")
    ctx.rhs_regular_box(Ss, dSs, (0, 0, 0), (7, 7, 7), dx, flags)
    n = (512, 256, 64)
    Sb = _periodic_grown(core, n)
    dSb = torch.full((5, n[2], n[1], n[0]), float("nan"), dtype=torch.float64, device="cuda")
    ctx.rhs_regular_box(Sb, dSb, (0, 0, 0), (n[0] - 1, n[1] - 1, n[2] - 1), dx, flags)
    torch.cuda.synchronize()
    assert bool(torch.isfinite(dSs).all())
    assert torch.equal(dSb, dSs.repeat(1, n[2] // 8, n[1] // 8, n[0] // 8))


@pytest.mark.parametrize("visc", [False, True])
def test_gravity_vs_oracle(ctx, oracle, visc):
    """EBR::do_gravity (Source/Advance.cpp:331-342): dSdt(UMZ) += g rho and
    dSdt(UEDEN) += g rho w after divop, g = -9.8; FP64 to 1e-12 and the mixed
    form's divergence plus the same FP64 source"""
    import ocfd
    S = inputs.ideal_state(20, 12, 10, 11)
    S = S.copy(); S[0] *= 1.2; S[1:4] *= 360.0; S[4] *= 1.0e5       # dimensional: g rho matters
    dxinv = [1.0e3, 1.1e3, 0.9e3]
    ref, _ = oracle.rhs_regular(S, dxinv, do_visc=visc, do_gravity=True)
    nog, _ = oracle.rhs_regular(S, dxinv, do_visc=visc)
    assert np.abs(ref[3] - nog[3]).max() > 0
    dS, _ = run_gpu(ctx, S, (3, -2, 0), dxinv, flags=int(visc) | ocfd.GRAVITY)
    for n in range(5):
        assert relerr(dS[n], ref[n]) < TOL, n
    d32, _ = run_gpu(ctx, S, (3, -2, 0), dxinv, flags=int(visc) | ocfd.GRAVITY | ocfd.FLUX_FP32)
    d32n, _ = run_gpu(ctx, S, (3, -2, 0), dxinv, flags=int(visc) | ocfd.FLUX_FP32)
    grav = ref - nog
    assert np.allclose(d32 - d32n, grav, rtol=1e-12, atol=1e-12 * np.abs(grav).max())
