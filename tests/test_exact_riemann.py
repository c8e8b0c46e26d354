"""The exact Riemann solver the Sod parity test measures L1 errors against:
Toro's star state for his test 1 (the Sod problem: p* = 0.30313, u* = 0.92745,
E. F. Toro, Riemann Solvers and Numerical Methods for Fluid Dynamics, table 4.3)
and the far-field / plateau states of the sampled solution."""
import numpy as np
import pytest

from exact_riemann import sample, star_state


def test_sod_star_state():
    p, u = star_state(1.0, 0.0, 1.0, 0.125, 0.0, 0.1)
    assert p == pytest.approx(0.30313, abs=1e-5)
    assert u == pytest.approx(0.92745, abs=1e-5)


def test_sod_sampled_profile():
    x = np.array([0.0, 0.3, 0.6, 0.75, 0.9, 1.0])
    r, u, p = sample(x, 0.2, 0.5, (1.0, 0.0, 1.0), (0.125, 0.0, 0.1))
    assert (r[0], u[0], p[0]) == (1.0, 0.0, 1.0)          # left of the rarefaction head
    assert (r[-1], u[-1], p[-1]) == (0.125, 0.0, 0.1)     # right of the shock
    assert p[2] == pytest.approx(0.30313, abs=1e-5)       # left star region
    assert r[3] == pytest.approx(0.26557, abs=1e-5)       # right star region (behind the shock)
    assert np.all(np.diff(r[:3]) <= 0)                    # density falls through the fan
