"""Exact solution of the 1D Riemann problem of the Euler equations for an ideal
gas (test infrastructure): the two-rarefaction / two-shock pressure function
solved by Newton's method for the star pressure, then sampled along x/t.
Method: E. F. Toro, "Riemann Solvers and Numerical Methods for Fluid
Dynamics", 3rd ed., ch. 4 (sec. 4.2-4.5).  Used for the L1 error of the Sod
shock tube (Exec/0_SOD/prob.H:13-38) against the exact solution."""
from __future__ import annotations

import math

import numpy as np


def _f(p, rho, pk, ck, g):
    """Toro eq. 4.6-4.7: the pressure function of one side and its derivative."""
    if p > pk:   # shock
        A = 2.0 / ((g + 1.0) * rho)
        B = (g - 1.0) / (g + 1.0) * pk
        s = math.sqrt(A / (B + p))
        return (p - pk) * s, s * (1.0 - 0.5 * (p - pk) / (B + p))
    r = p / pk   # rarefaction
    return 2.0 * ck / (g - 1.0) * (r ** ((g - 1.0) / (2.0 * g)) - 1.0), \
        1.0 / (rho * ck) * r ** (-(g + 1.0) / (2.0 * g))


def star_state(rl, ul, pl, rr, ur, pr, g=1.4):
    cl, cr = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)
    p = max(1e-12, 0.5 * (pl + pr) - 0.125 * (ur - ul) * (rl + rr) * (cl + cr))
    for _ in range(100):
        fl, dl = _f(p, rl, pl, cl, g)
        fr, dr = _f(p, rr, pr, cr, g)
        pn = max(1e-12, p - (fl + fr + ur - ul) / (dl + dr))
        if abs(pn - p) <= 1e-15 * 0.5 * (pn + p):
            p = pn
            break
        p = pn
    fl, _ = _f(p, rl, pl, cl, g)
    fr, _ = _f(p, rr, pr, cr, g)
    return p, 0.5 * (ul + ur) + 0.5 * (fr - fl)


def sample(x, t, x0, left, right, g=1.4):
    """(rho, u, p) at positions x, time t, for the states left / right =
    (rho, u, p) separated at x0 (Toro sec. 4.5)."""
    rl, ul, pl = left
    rr, ur, pr = right
    ps, us = star_state(rl, ul, pl, rr, ur, pr, g)
    cl, cr = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)
    gm = (g - 1.0) / (g + 1.0)
    out = np.empty((3, len(x)))
    for i, xi in enumerate(x):
        s = (xi - x0) / t
        if s <= us:   # left of the contact
            if ps > pl:
                sl = ul - cl * math.sqrt((g + 1.0) / (2.0 * g) * ps / pl + (g - 1.0) / (2.0 * g))
                st = (rl * (ps / pl + gm) / (gm * ps / pl + 1.0), us, ps) if s >= sl else (rl, ul, pl)
            else:
                csl = cl * (ps / pl) ** ((g - 1.0) / (2.0 * g))
                if s <= ul - cl:
                    st = (rl, ul, pl)
                elif s >= us - csl:
                    st = (rl * (ps / pl) ** (1.0 / g), us, ps)
                else:
                    c = 2.0 / (g + 1.0) * (cl + 0.5 * (g - 1.0) * (ul - s))
                    u = 2.0 / (g + 1.0) * (cl + 0.5 * (g - 1.0) * ul + s)
                    st = (rl * (c / cl) ** (2.0 / (g - 1.0)), u, pl * (c / cl) ** (2.0 * g / (g - 1.0)))
        else:
            if ps > pr:
                sr = ur + cr * math.sqrt((g + 1.0) / (2.0 * g) * ps / pr + (g - 1.0) / (2.0 * g))
                st = (rr * (ps / pr + gm) / (gm * ps / pr + 1.0), us, ps) if s <= sr else (rr, ur, pr)
            else:
                csr = cr * (ps / pr) ** ((g - 1.0) / (2.0 * g))
                if s >= ur + cr:
                    st = (rr, ur, pr)
                elif s <= us + csr:
                    st = (rr * (ps / pr) ** (1.0 / g), us, ps)
                else:
                    c = 2.0 / (g + 1.0) * (cr - 0.5 * (g - 1.0) * (ur - s))
                    u = 2.0 / (g + 1.0) * (-cr + 0.5 * (g - 1.0) * ur + s)
                    st = (rr * (c / cr) ** (2.0 / (g - 1.0)), u, pr * (c / cr) ** (2.0 * g / (g - 1.0)))
        out[:, i] = st
    return out
