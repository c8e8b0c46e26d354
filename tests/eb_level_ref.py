"""CPU reference of a level cut by an embedded body: the box loop of
EBR::compute_dSdt (Source/Advance.cpp:201-342) - covered box -> zero RHS, box
whose grow(bx, 4) is all regular -> regular WENO-Z RHS, any other box -> the
cut-cell RHS of eb_compute_dSdt_box - inside the oracle's SSP-RK3 (Shu-Osher)
step with its ghost fill and CFL step, on whole-level arrays.

Both RHS are evaluated over the whole level and selected per cell by the class
of the cell's box: every RHS value depends only on the state and geometry in a
few cells around it, so this equals the per-box evaluation.  Test
infrastructure only."""
from __future__ import annotations

import numpy as np

from oracle import BCStruct, NG

T_REGULAR, T_CUT, T_COVERED = 0, 1, 3
BOX_REGULAR, BOX_CUT, BOX_COVERED = 0, 1, 2


def box_classes(geom, boxes):
    """class of each box from the level geometry (arrays over the domain grown by NG)"""
    typ = geom["flag"][0] & 3
    out = []
    for lo, hi in boxes:
        valid = typ[NG + lo[2]:NG + hi[2] + 1, NG + lo[1]:NG + hi[1] + 1, NG + lo[0]:NG + hi[0] + 1]
        grown = typ[lo[2]:hi[2] + 2 * NG + 1, lo[1]:hi[1] + 2 * NG + 1, lo[0]:hi[0] + 2 * NG + 1]
        if np.all(valid == T_COVERED):
            out.append(BOX_COVERED)
        elif np.all(grown == T_REGULAR):
            out.append(BOX_REGULAR)
        else:
            out.append(BOX_CUT)
    return out


def cell_class(classes, boxes, n):
    c = np.zeros((n[2], n[1], n[0]), dtype=np.int32)
    for cl, (lo, hi) in zip(classes, boxes):
        c[lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] = cl
    return c


def make_bc(case):
    bc = BCStruct()
    bc.lo_bc[:] = list(case["lo_bc"])
    bc.hi_bc[:] = list(case["hi_bc"])
    bc.dirichlet_case = case.get("bc_case", 0)
    bc.prob_lo[:] = list(case["prob_lo"])
    bc.dx[:] = list(case["dx"])
    bc.dom_lo[:] = [0, 0, 0]
    bc.dom_hi[:] = [m - 1 for m in case["n"]]
    if bc.dirichlet_case == 3:
        bc.jet[:] = list(case["case_params"][:8])
    return bc


def advance(oracle, case, geom, classes, boxes, nsteps, cfl, visc=False, redist=False):
    """nsteps SSP-RK3 steps of the whole level; returns (valid state, time)."""
    n = case["n"]
    S = np.ascontiguousarray(case["G"].copy())
    bc = make_bc(case)
    dx = case["dx"]
    dxinv = tuple(1.0 / d for d in dx)
    cc = cell_class(classes, boxes, n)[None]
    inner = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))

    def rhs(U):
        with np.errstate(all="ignore"):
            dr, _ = oracle.rhs_regular(U, dxinv, do_visc=visc)
            de, _ = oracle.rhs_eb(U, geom, dxinv, do_visc=visc, do_redistribute=redist)
        return np.where(cc == BOX_REGULAR, dr, np.where(cc == BOX_CUT, de, 0.0))

    t, dt_prev = 0.0, -1.0
    for _ in range(nsteps):
        oracle.fill_ghosts(bc, S, t)
        dt = cfl * oracle.estdt(S, dx)
        if dt_prev > 0 and dt > 1.1 * dt_prev:
            dt = 1.1 * dt_prev
        dt_prev = dt
        S0 = S.copy()
        k1 = rhs(S)
        Ss = S0.copy()
        Ss[inner] = S0[inner] + dt * k1
        oracle.fill_ghosts(bc, Ss, t + dt)
        k2 = rhs(Ss)
        Ss[inner] = 0.75 * S0[inner] + 0.25 * (Ss[inner] + dt * k2)
        oracle.fill_ghosts(bc, Ss, t + 0.5 * dt)
        k3 = rhs(Ss)
        S[inner] = (1.0 / 3.0) * S0[inner] + (2.0 / 3.0) * (Ss[inner] + dt * k3)
        t += dt
    return S[inner].copy(), t


def uniform_flow(n, rho=1.4, p=1.0, u=2.0, gamma=1.4):
    """uniform state over the grown level (u along x)"""
    sh = (n[2] + 2 * NG, n[1] + 2 * NG, n[0] + 2 * NG)
    G = np.empty((5,) + sh)
    G[0] = rho
    G[1] = rho * u
    G[2] = 0.0
    G[3] = 0.0
    G[4] = p / (gamma - 1) + 0.5 * rho * u * u
    return G
