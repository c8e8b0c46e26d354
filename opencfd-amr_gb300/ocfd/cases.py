"""Initial conditions and boundary setups of the benchmark configurations
(fixtures; Exec/<case>/prob.H restated), on a global grown array
(5, Nz+8, Ny+8, Nx+8) whose first cell is (-4, -4, -4)."""
from __future__ import annotations

import math

import numpy as np

NG = 4
GAMMA = 1.4


def _centres(n, dx, prob_lo):
    return [prob_lo[d] + (np.arange(-NG, n[d] + NG) + 0.5) * dx[d] for d in range(3)]


def sod(nx=512, ny=64, nz=4, gamma=GAMMA):
    """2D Sod shock tube on [0,1] x [0,0.125] as a thin slab (Exec/0_SOD/prob.H:13-38,
    prob_parm.H:9-12).  BCs of Exec/0_SOD/inputs:15-16: x outflow, y and z slip walls."""
    dx = 1.0 / nx
    n = (nx, ny, nz)
    x, _, _ = _centres(n, (dx, dx, dx), (0.0, 0.0, 0.0))
    G = np.zeros((5, nz + 2 * NG, ny + 2 * NG, nx + 2 * NG))
    left = x < 0.5
    rho = np.where(left, 1.0, 0.125)
    p = np.where(left, 1.0, 0.1)
    G[0] = rho[None, None, :]
    G[4] = (p / (gamma - 1.0))[None, None, :]
    return dict(G=G, n=n, dx=(dx, dx, dx), prob_lo=(0.0, 0.0, 0.0),
                lo_bc=(2, 4, 4), hi_bc=(2, 4, 4), bc_case=0, case_params=())


def dmr_states(gamma=GAMMA):
    """Post-shock (left) and pre-shock (right) conserved states, Exec/1_DMR/prob_parm.H:10-17."""
    rl, pl = 8.0, 116.5
    ul, vl = 8.25 * math.cos(math.pi / 6.0), -8.25 * math.sin(math.pi / 6.0)
    rr, pr = 1.4, 1.0
    left = [rl, rl * ul, rl * vl, 0.0, pl / (gamma - 1.0) + 0.5 * rl * (ul * ul + vl * vl)]
    right = [rr, 0.0, 0.0, 0.0, pr / (gamma - 1.0)]
    return left, right


def dmr(nx=1024, ny=256, nz=2, gamma=GAMMA, Lx=4.0):
    """Double Mach reflection on [0,4] x [0,1] (Exec/1_DMR/prob.H:11-46), thin in z.
    BCs of Exec/1_DMR/inputs:15-16: x inflow/outflow, y slip wall / inflow, z outflow."""
    dx = Lx / nx
    n = (nx, ny, nz)
    x, y, _ = _centres(n, (dx, dx, dx), (0.0, 0.0, 0.0))
    left, right = dmr_states(gamma)
    X, Y = np.meshgrid(x, y, indexing="xy")          # (ny+8, nx+8)
    post = X < 1.0 / 6.0 + math.sqrt(1 / 3.0) * Y
    G = np.zeros((5, nz + 2 * NG, ny + 2 * NG, nx + 2 * NG))
    for c in range(5):
        G[c] = np.where(post, left[c], right[c])[None]
    return dict(G=G, n=n, dx=(dx, dx, dx), prob_lo=(0.0, 0.0, 0.0),
                lo_bc=(1, 4, 2), hi_bc=(2, 1, 2), bc_case=1, case_params=tuple(left) + tuple(right))


def blast3d(nx=256, ny=256, nz=64, gamma=GAMMA):
    """3D periodic blast: rho=1, p=1 inside r < 0.2 of the box centre, 0.125 / 0.1
    outside; unit cell size 1/nx.  A regular-box workload larger than L2."""
    dx = 1.0 / nx
    n = (nx, ny, nz)
    x, y, z = _centres(n, (dx, dx, dx), (0.0, 0.0, 0.0))
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    r = np.sqrt((X - 0.5 * nx * dx) ** 2 + (Y - 0.5 * ny * dx) ** 2 + (Z - 0.5 * nz * dx) ** 2)
    inside = r < 0.2 * min(n) * dx
    G = np.zeros((5, nz + 2 * NG, ny + 2 * NG, nx + 2 * NG))
    G[0] = np.where(inside, 1.0, 0.125)
    G[4] = np.where(inside, 1.0, 0.1) / (gamma - 1.0)
    return dict(G=G, n=n, dx=(dx, dx, dx), prob_lo=(0.0, 0.0, 0.0),
                lo_bc=(0, 0, 0), hi_bc=(0, 0, 0), bc_case=0, case_params=())


def dmr_fab(lo, hi, dx, gamma=GAMMA):
    """Grown FAB (5, nz+8, ny+8, nx+8) of the DMR initial condition over the box
    lo..hi at cell size dx (Exec/1_DMR/prob.H:11-46)."""
    x = (np.arange(lo[0] - NG, hi[0] + NG + 1) + 0.5) * dx[0]
    y = (np.arange(lo[1] - NG, hi[1] + NG + 1) + 0.5) * dx[1]
    nz = hi[2] - lo[2] + 1 + 2 * NG
    left, right = dmr_states(gamma)
    X, Y = np.meshgrid(x, y, indexing="xy")
    post = X < 1.0 / 6.0 + math.sqrt(1 / 3.0) * Y
    F = np.empty((5, nz, len(y), len(x)))
    for c in range(5):
        F[c] = np.where(post, left[c], right[c])[None]
    return F


def dmr_amr(nx=1024, ny=256, nz=2, max_level=2, blocking_factor=32, max_grid=128, n_error_buf=1,
            refine_dengrad=0.05, regrid_int=2, gamma=GAMMA, Lx=4.0):
    """Double Mach reflection with refinement: base nx x ny x nz, ratio 2,
    |d rho| >= refine_dengrad tagging (Exec/1_DMR/inputs:48-49), blocking factor
    and max grid size in cells of each level (z blocks span the thin slab)."""
    dx = Lx / nx
    left, right = dmr_states(gamma)
    return dict(n=(nx, ny, nz), dx=(dx, dx, dx), prob_lo=(0.0, 0.0, 0.0), lo_bc=(1, 4, 2), hi_bc=(2, 1, 2),
                bc_case=1, case_params=tuple(left) + tuple(right), max_level=max_level,
                blocking_factor=(blocking_factor,) * 3, max_grid_size=(max_grid,) * 3,
                n_error_buf=n_error_buf, refine_dengrad=refine_dengrad, regrid_int=regrid_int,
                fab=lambda lev, lo, hi, d: dmr_fab(lo, hi, d, gamma))


JET_SEED = 20261203


def jet_params(gamma=GAMMA, rho=1.4, p=1.0, mach=2.0, u_co=0.5, yc=0.5, half_width=0.25, delta=0.02,
               rho_co=1.0):
    """Inflow parameters of the planar jet (OCFD_CASE_JET): rho_jet, u_jet, u_co,
    yc, w, delta, rho e, rho_co.  rho = 1.4, p = 1 gives c = 1 in the jet, so
    u_jet = Mach number; the co-flow is lighter (rho_co) and slower (u_co c)."""
    c = math.sqrt(gamma * p / rho)
    return (rho, mach * c, u_co * c, yc, half_width, delta, p / (gamma - 1.0), rho_co)


def jet_kh_modes(seed=JET_SEED, nx_modes=4, nz_modes=3):
    """Random phases of the Kelvin-Helmholtz perturbation modes (x mode m =
    1..nx_modes, z mode l = 0..nz_modes-1), numpy PCG64 seeded with `seed`."""
    rng = np.random.default_rng(seed)
    return rng.uniform(0.0, 2.0 * math.pi, size=(nx_modes, nz_modes))


def jet_fab(lo, hi, dx, prob_lo=(0.0, 0.0, 0.0), L=(2.0, 1.0, 1.0), params=None, amp=1e-2, seed=JET_SEED,
            gamma=GAMMA, thickness=None):
    """Grown FAB (5, nz+8, ny+8, nx+8) of the jet initial condition over lo..hi:
    the inflow profile everywhere plus a transverse velocity perturbation
    v' = amp u_jet sum_{m,l} sin(2 pi (m x / Lx + l z / Lz) + phi_ml) g(y) / (M L)
    concentrated on the two shear layers, g(y) = sum_+- exp(-((y - yc -+ w) / (4 delta))^2)."""
    rho_j, uj, uc, yc, w, delta, rhoe, rho_c = params if params is not None else jet_params(gamma)
    x = prob_lo[0] + (np.arange(lo[0] - NG, hi[0] + NG + 1) + 0.5) * dx[0]
    y = prob_lo[1] + (np.arange(lo[1] - NG, hi[1] + NG + 1) + 0.5) * dx[1]
    z = prob_lo[2] + (np.arange(lo[2] - NG, hi[2] + NG + 1) + 0.5) * dx[2]
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    sh = 0.5 * (1.0 + np.tanh((w - np.abs(Y - yc)) / delta))
    u = uc + (uj - uc) * sh
    rho = rho_c + (rho_j - rho_c) * sh
    th = 4.0 * delta if thickness is None else thickness
    g = np.exp(-((Y - yc - w) / th) ** 2) + np.exp(-((Y - yc + w) / th) ** 2)
    ph = jet_kh_modes(seed)
    M, Lm = ph.shape
    v = np.zeros_like(X)
    for m in range(M):
        for l in range(Lm):
            v += np.sin(2 * math.pi * ((m + 1) * X / L[0] + l * Z / L[2]) + ph[m, l])
    v *= amp * uj * g / (M * Lm)
    F = np.empty((5,) + X.shape)
    F[0] = rho
    F[1] = rho * u
    F[2] = rho * v
    F[3] = 0.0
    F[4] = rhoe + 0.5 * rho * (u * u + v * v)
    return F


def jet_eb_amr(nx=256, ny=128, nz=128, max_level=2, blocking_factor=8, max_grid=64, n_error_buf=1,
               refine_dengrad=0.1, regrid_int=2, gamma=GAMMA, center=(0.5, 0.5), radius=0.1, redistribute=True):
    """Mach 2 planar jet past a z-aligned cylinder (radius 0.1 at (0.5, 0.5)) in
    [0,2] x [0,1] x [0,1]: x-lo jet inflow (OCFD_CASE_JET), x-hi and y outflow,
    z periodic; Kelvin-Helmholtz perturbations of amplitude 1e-2 with seeded
    random phases on the shear layers; ratio-2 levels tagged by |d rho|.  The
    cut cells use the reference's small-cell rescale (ebr.do_redistribute = 1,
    Source/EB/EBkernels.H:341-377): without it the unscaled 1/vfrac update of
    cells with small volume fractions is unstable at CFL 0.5."""
    dx = 2.0 / nx
    params = jet_params(gamma)
    return dict(n=(nx, ny, nz), dx=(dx, dx, dx), prob_lo=(0.0, 0.0, 0.0), lo_bc=(1, 2, 0), hi_bc=(2, 2, 0),
                bc_case=3, case_params=params, max_level=max_level, blocking_factor=(blocking_factor,) * 3,
                max_grid_size=(max_grid,) * 3, n_error_buf=n_error_buf, refine_dengrad=refine_dengrad,
                regrid_int=regrid_int, eb=dict(center=center, radius=radius, redistribute=redistribute), seed=JET_SEED,
                fab=lambda lev, lo, hi, d: jet_fab(lo, hi, d, L=(nx * dx, ny * dx, nz * dx), params=params,
                                                   gamma=gamma))


def jet_eb(nx=256, ny=128, nz=128, gamma=GAMMA, center=(0.5, 0.5), radius=0.1, redistribute=True):
    """Single-level form of jet_eb_amr on a global grown array."""
    c = jet_eb_amr(nx, ny, nz, gamma=gamma, center=center, radius=radius, redistribute=redistribute)
    n = c["n"]
    G = jet_fab((0, 0, 0), (n[0] - 1, n[1] - 1, n[2] - 1), c["dx"], L=tuple(m * c["dx"][0] for m in n),
                params=c["case_params"], gamma=gamma)
    return dict(G=G, n=n, dx=c["dx"], prob_lo=c["prob_lo"], lo_bc=c["lo_bc"], hi_bc=c["hi_bc"], bc_case=3,
                case_params=c["case_params"], eb=c["eb"])


# Species order of the mechanism: H2, O2, H2O, H, O, OH, HO2, H2O2, N2
PHI1_AIR_X = (0.2958, 0.1479, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.5563)


def hot_spot_temperature(n=128, length=0.01, seed=20261203, nspots=8, t0=1200.0, dT=600.0, radius_cells=6.0):
    """Temperature over the grown periodic box (nz+8, ny+8, nx+8): t0 plus 8
    Gaussian hot spots dT * exp(-(r / (6 dx))^2) at centres drawn from
    MT19937(seed), periodic minimum-image distances."""
    dx = length / n
    rng = np.random.Generator(np.random.MT19937(seed))
    centres = rng.uniform(0.0, length, size=(nspots, 3))
    x = (np.arange(-NG, n + NG) + 0.5) * dx
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    T = np.full(Z.shape, t0)
    for cx, cy, cz in centres:
        d2 = 0.0
        for coord, c in ((X, cx), (Y, cy), (Z, cz)):
            d = np.abs(coord - c)
            d = np.minimum(d, length - d)
            d2 = d2 + d * d
        T += dT * np.exp(-d2 / (radius_cells * dx) ** 2)
    return T, dx, centres


def react_cube(ctx, n=128, length=0.01, seed=20261203, p=101325.0):
    """The reacting workload: premixed phi = 1 H2/air at 1 atm, 1200 K with 8 seeded hot
    spots, periodic cube of n^3 cells and edge `length`; the grown global state
    (14, n+8, n+8, n+8): conserved variables then partial densities."""
    from .react import state_tpx
    T, dx, centres = hot_spot_temperature(n, length, seed)
    X = np.array(PHI1_AIR_X)[:, None, None, None] * np.ones((1,) + T.shape)
    G = state_tpx(ctx, T, p, X)
    return dict(G=G, n=(n, n, n), dx=(dx, dx, dx), T=T, centres=centres, seed=seed, length=length)
