"""Seeded synthetic inputs for the parity tests (numpy's PCG64, so the same seed
gives the same arrays on every machine).

States are physical (positive density and pressure) but deliberately rough:
smooth waves plus jumps, sub- and supersonic velocities of both signs, so that
every branch of the Steger-Warming split, the WENO-Z weights, the Van Leer flux
and the minmod limiter is exercised.
"""
from __future__ import annotations

import os
import sys

import numpy as np

NG = 4
NSPEC = 9
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "opencfd-amr_gb300"))


def grown(nc, nx, ny, nz):
    return (nc, nz + 2 * NG, ny + 2 * NG, nx + 2 * NG)


def ideal_state(nx, ny, nz, seed, gamma=1.4, mach=1.5, jump=True):
    """Conserved ideal-gas state over the grown box."""
    rng = np.random.default_rng(seed)
    sh = grown(1, nx, ny, nz)[1:]
    z, y, x = np.meshgrid(*[np.linspace(0, 1, s) for s in sh], indexing="ij")
    rho = 1.0 + 0.3 * np.sin(2 * np.pi * (x + 0.7 * y) + rng.random()) + 0.2 * rng.random(sh)
    p = 1.0 + 0.4 * np.cos(2 * np.pi * (y - 0.4 * z) + rng.random()) + 0.2 * rng.random(sh)
    if jump:
        cut = x + 0.3 * y > 0.55
        rho = np.where(cut, 0.125 * rho, rho)
        p = np.where(cut, 0.1 * p, p)
    c = np.sqrt(gamma * p / rho)
    u = mach * c * (rng.standard_normal((3,) + sh) * 0.6 + 0.3 * np.sin(6 * x)[None])
    S = np.empty(grown(5, nx, ny, nz))
    S[0] = rho
    S[1:4] = rho * u
    S[4] = p / (gamma - 1) + 0.5 * rho * (u * u).sum(0)
    return S


def chem_state(nx, ny, nz, seed, oracle, T_range=(300.0, 2600.0), p0=101325.0, vel=300.0):
    """Conserved state + species partial densities for H2/O2/N2 mixtures with
    products and radicals.  Energy from the oracle's CKUBMS so that T is
    recovered by the Newton inversion."""
    rng = np.random.default_rng(seed)
    sh = grown(1, nx, ny, nz)[1:]
    ncell = int(np.prod(sh))
    T = rng.uniform(*T_range, size=ncell)
    p = p0 * rng.uniform(0.7, 1.3, size=ncell)
    X = np.zeros((ncell, NSPEC))
    X[:, 0] = rng.uniform(0.05, 0.35, ncell)   # H2
    X[:, 1] = rng.uniform(0.05, 0.2, ncell)    # O2
    X[:, 2] = rng.uniform(0.0, 0.2, ncell)     # H2O
    X[:, 3:8] = rng.uniform(0.0, 0.01, (ncell, 5)) * (rng.random((ncell, 5)) < 0.7)
    X[:, 8] = 1.0 - X[:, :8].sum(1)            # N2
    rho = np.empty(ncell)
    rhoi = np.empty((ncell, NSPEC))
    e = np.empty(ncell)
    for c in range(ncell):
        Y = oracle.ckxty(X[c])
        rho[c] = oracle.ckrhoy(p[c], T[c], Y)
        rhoi[c] = rho[c] * Y
        e[c] = oracle.ckubms(T[c], rhoi[c])
    u = vel * rng.standard_normal((3, ncell))
    S = np.empty((5, ncell))
    S[0] = rho
    S[1:4] = rho * u
    S[4] = e + 0.5 * rho * (u * u).sum(0)
    spec = np.ascontiguousarray(rhoi.T)
    return S.reshape(grown(5, nx, ny, nz)).copy(), spec.reshape(grown(NSPEC, nx, ny, nz)).copy()


def cylinder_box(nx, ny, nz, lo=(0, 0, 0), r_cells=None, center_cells=None):
    """EB geometry of a box cut by a z-aligned cylinder (unit cell size)."""
    from ocfd.geometry import box_geometry, cylinder_phi
    if center_cells is None:
        center_cells = (lo[0] + nx * 0.45, lo[1] + ny * 0.55)
    if r_cells is None:
        r_cells = 0.3 * min(nx, ny)
    phi = cylinder_phi(center_cells[0], center_cells[1], r_cells)
    return box_geometry(phi, lo, (nx, ny, nz), (1.0, 1.0, 1.0), nsub=16)


def react_hot_spot_fab(oracle, n_domain, dx, T0=1200.0, dT=600.0, radius_cells=3.0, p=101325.0):
    """fab_of_box(lev, lo, hi, dx_l) for a periodic phi = 1 H2/air box with one
    Gaussian hot spot at the domain centre (radius in level-0 cells): the grown
    FAB (14, nz+8, ny+8, nx+8) of conserved state and partial densities,
    built on the host with the oracle's CKXTY / CKRHOY / CKUBMS."""
    from ocfd.cases import PHI1_AIR_X
    y = oracle.ckxty(np.array(PHI1_AIR_X))
    L = [n * dx for n in n_domain]
    centre = [0.5 * x for x in L]
    cache = {}

    def fab(lev, lo, hi, dxl):
        key = (lev, tuple(lo), tuple(hi))
        if key in cache:
            return cache[key].copy()
        coords = [(np.arange(lo[d] - NG, hi[d] + NG + 1) + 0.5) * dxl[d] for d in range(3)]
        Z, Y, X = np.meshgrid(coords[2], coords[1], coords[0], indexing="ij")
        r2 = 0.0
        for C, c, Ld in ((X, centre[0], L[0]), (Y, centre[1], L[1]), (Z, centre[2], L[2])):
            dd = np.abs(np.mod(C, Ld) - c)
            dd = np.minimum(dd, Ld - dd)
            r2 = r2 + dd * dd
        T = T0 + dT * np.exp(-r2 / (radius_cells * dx) ** 2)
        F = np.zeros((5 + NSPEC,) + T.shape)
        flat = T.ravel()
        for i, t in enumerate(flat):
            idx = np.unravel_index(i, T.shape)
            rho = oracle.ckrhoy(p, float(t), y)
            r = rho * y
            F[(0,) + idx] = rho
            F[(4,) + idx] = oracle.ckubms(float(t), r)
            F[(slice(5, None),) + idx] = r
        cache[key] = F
        return F.copy()
    return fab
