"""The whole-level cut-cell reference used by the GPU tests, checked on the CPU:
box classes of a known geometry, and - with no body - bit-identity with the
oracle's own SSP-RK3 driver (ocfdo_advance_rk3, Shu-Osher form)."""
import numpy as np

import eb_level_ref as ref
from oracle import NG


def test_box_classes_of_a_cylinder():
    from ocfd import geometry
    n, dx = (64, 64, 2), (1 / 64,) * 3
    g = geometry.box_geometry(geometry.cylinder_phi(0.25, 0.25, 0.2), (0, 0, 0), n, dx)
    boxes = [((i, j, 0), (i + 7, j + 7, 1)) for j in range(0, 64, 8) for i in range(0, 64, 8)]
    cls = ref.box_classes(g, boxes)
    c, r = 16.0, 12.8   # centre and radius in cells
    for b, (lo, hi) in enumerate(boxes):
        far = [max(abs(lo[d] - c), abs(hi[d] + 1 - c)) for d in (0, 1)]
        near = [max(lo[d] - 4 - c, c - (hi[d] + 5), 0.0) for d in (0, 1)]
        if np.hypot(*far) < r:
            assert cls[b] == ref.BOX_COVERED, b
        elif np.hypot(*near) > r:
            assert cls[b] == ref.BOX_REGULAR, b
        else:
            assert cls[b] == ref.BOX_CUT, b
    assert set(cls) == {0, 1, 2}


def test_no_body_equals_the_oracle_driver(oracle):
    from ocfd import geometry
    n = (24, 16, 4)
    dx = (1 / 24,) * 3
    rng = np.random.default_rng(5)
    G = ref.uniform_flow(n) * (1 + 0.05 * rng.standard_normal((5, n[2] + 8, n[1] + 8, n[0] + 8)))
    case = dict(n=n, dx=dx, prob_lo=(0, 0, 0), lo_bc=(2, 4, 0), hi_bc=(2, 4, 0), bc_case=0, G=G)
    g = geometry.box_geometry(geometry.cylinder_phi(-5.0, -5.0, 0.1), (0, 0, 0), n, dx)
    boxes = [((0, 0, 0), (11, 15, 3)), ((12, 0, 0), (23, 15, 3))]
    cls = ref.box_classes(g, boxes)
    assert cls == [ref.BOX_REGULAR] * 2
    got, t = ref.advance(oracle, case, g, cls, boxes, 3, 0.5)
    S = np.ascontiguousarray(G.copy())
    t2, _ = oracle.advance_rk3(ref.make_bc(case), S, 0.5, 3, form=1)
    assert t == t2
    assert np.array_equal(got, S[:, NG:-NG, NG:-NG, NG:-NG])


def test_fixture_geometry_measures_the_cylinder():
    """The sub-sampled geometry (the fixture the device geometry must equal):
    the covered area is the disc's area to the sampling resolution, the area
    fractions of the faces crossing the circle lie strictly between 0 and 1,
    and a cell is regular exactly when its volume fraction and its four face
    fractions are 1."""
    from ocfd import geometry
    n, dx, r = (48, 48, 1), (1 / 48,) * 3, 0.3
    g = geometry.box_geometry(geometry.cylinder_phi(0.5, 0.5, r), (0, 0, 0), n, dx, nsub=16)
    vf = g["vfrac"][0, NG, NG:-NG, NG:-NG]
    covered_area = float((1.0 - vf).sum()) * dx[0] * dx[1]
    assert abs(covered_area - np.pi * r * r) < 2e-3
    apx = g["apx"][0, 0]
    assert ((apx > 0) & (apx < 1)).any()
    typ = g["flag"][0, NG, NG:-NG, NG:-NG] & 3
    full = (vf == 1.0) & (apx[:, :-1] == 1.0) & (apx[:, 1:] == 1.0) & \
        (g["apy"][0, 0][:-1, :] == 1.0) & (g["apy"][0, 0][1:, :] == 1.0)
    assert np.array_equal(typ == 0, full)
