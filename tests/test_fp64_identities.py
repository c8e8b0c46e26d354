"""The identities the FP64 kernels' arithmetic rests on, checked on the CPU in
numpy float64 against the reference's expressions:

- WENO-Z (Source/kernel/Reconstruction.H:83-138) with the smoothness indicators
  carried as 4 beta, the weights from one triple product and the 1/6 and linear
  weights folded into the candidate polynomials (device_physics.cuh
  wenoz_face_e): the same face values up to rounding;
- the Steger-Warming split (Source/kernel/FluxSplit.H:11-193) regrouped as in
  device_physics.cuh sw_split_d: the same fluxes up to rounding, with the
  eigenvalue parts exactly max(x, 0) and min(x, 0);
- the CFL bound (Source/Advance.cpp:26-49): the minimum over cells of dx / s is
  exactly dx / max s, because a correctly rounded division is monotone in its
  divisor (rhs_regular.h CflSpeeds reduces the largest speeds per block).

These restate the kernels' formulas in numpy (no FMA); the kernels themselves are
checked against the oracle by the -m gpu parity tests."""
import numpy as np


def wenoz_ref(V1, V2, V3, V4, V5):
    eps = 1e-6
    s11 = (13.0 / 12.0) * (V1 - 2.0 * V2 + V3) * (V1 - 2.0 * V2 + V3) + \
        0.25 * (V1 - 4.0 * V2 + 3.0 * V3) * (V1 - 4.0 * V2 + 3.0 * V3)
    s22 = (13.0 / 12.0) * (V2 - 2.0 * V3 + V4) * (V2 - 2.0 * V3 + V4) + 0.25 * (V2 - V4) * (V2 - V4)
    s33 = (13.0 / 12.0) * (V3 - 2.0 * V4 + V5) * (V3 - 2.0 * V4 + V5) + \
        0.25 * (3.0 * V3 - 4.0 * V4 + V5) * (3.0 * V3 - 4.0 * V4 + V5)
    s55 = np.abs(s11 - s33)
    s11 = 1.0 + (s55 / (eps + s11)) * (s55 / (eps + s11))
    s22 = 1.0 + (s55 / (eps + s22)) * (s55 / (eps + s22))
    s33 = 1.0 + (s55 / (eps + s33)) * (s55 / (eps + s33))
    a1, a2, a3 = s11, 6.0 * s22, 3.0 * s33
    invsum = 1.0 / (a1 + a2 + a3)
    v1 = 2.0 * V1 - 7.0 * V2 + 11.0 * V3
    v2 = -V2 + 5.0 * V3 + 2.0 * V4
    v3 = 2.0 * V3 + 5.0 * V4 - V5
    return (1.0 / 6.0) * invsum * (a1 * v1 + a2 * v2 + a3 * v3)


def wenoz_folded(V1, V2, V3, V4, V5):
    def e2(a, b, c):
        e = (a - 2.0 * b) + c
        return ((13.0 / 3.0) * e) * e
    E1, E2, E3 = e2(V1, V2, V3), e2(V2, V3, V4), e2(V3, V4, V5)
    eps4 = 4e-6
    g1 = 3.0 * V3 + (V1 - 4.0 * V2)
    g2 = V2 - V4
    g3 = -4.0 * V4 + (3.0 * V3 + V5)
    b1, b2, b3 = g1 * g1 + E1, g2 * g2 + E2, g3 * g3 + E3
    tau = np.abs(b1 - b3)
    D1, D2, D3 = eps4 + b1, eps4 + b2, eps4 + b3
    q1, q2, q3, t2 = D1 * D1, D2 * D2, D3 * D3, tau * tau
    q12, q13, q23 = q1 * q2, q1 * q3, q2 * q3
    P = q12 * q3
    A1, A2, A3 = t2 * q23 + P, t2 * q13 + P, t2 * q12 + P
    c1 = (11.0 / 6.0) * V3 + ((-7.0 / 6.0) * V2 + (1.0 / 3.0) * V1)
    c2 = 2.0 * V4 + (5.0 * V3 - V2)
    c3 = -0.5 * V5 + (2.5 * V4 + V3)
    num = A3 * c3 + (A2 * c2 + A1 * c1)
    den = 3.0 * A3 + (6.0 * A2 + A1)
    return num / den


def lines(rng, n=4000, N=32):
    """Pencil lines of a split flux: smooth waves over a base, some with a jump,
    magnitudes from 1e-2 to 1e8 and amplitudes down to 1e-3 of the base."""
    base = 10.0 ** rng.uniform(-2, 8, (n, 1))
    amp = base * 10.0 ** rng.uniform(-3, 0, (n, 1))
    i = np.arange(N + 6)[None, :]
    V = base + amp * np.sin(2 * np.pi * i / N + rng.uniform(0, 2 * np.pi, (n, 1)))
    jump = rng.integers(0, N, (n, 1))
    V = V + np.where((i > jump) & (rng.uniform(size=(n, 1)) < 0.3), 0.5 * base, 0.0)
    return V


def faces(f, V):
    return f(V[:, :-5], V[:, 1:-4], V[:, 2:-3], V[:, 3:-2], V[:, 4:-1])


def test_wenoz_folded_matches_reference():
    rng = np.random.default_rng(20261204)
    V = lines(rng)
    r, g = faces(wenoz_ref, V), faces(wenoz_folded, V)
    scale = np.abs(V).max(axis=1, keepdims=True)
    # a few ulps of the stencil's magnitude (measured: 7e-16)
    assert (np.abs(g - r) / scale).max() < 1e-14
    # the flux divergence of a line, norm-wise against its own magnitude; lines
    # whose amplitude is 1e-3 of their base lose three digits in the difference
    # of neighbouring faces either way (measured: median 2e-14, max 4e-12)
    dr, dg = np.diff(r, axis=1), np.diff(g, axis=1)
    err = np.abs(dg - dr).max(axis=1) / np.abs(dr).max(axis=1)
    assert np.median(err) < 1e-13 and err.max() < 1e-10


def test_wenoz_folded_constant_and_linear_data():
    """Constant data reconstruct the constant, linear data the face value, to
    rounding; the scaled indicators keep every weight finite up to |V| ~ 1e12."""
    for c in (0.0, 1e-9, 1.0, 3.7e5, 2.5e12):
        V = np.full((1, 11), c)
        assert np.allclose(faces(wenoz_folded, V), c, rtol=1e-15, atol=0)
    x = np.arange(11, dtype=np.float64)[None, :]
    V = 2.0 + 0.125 * x
    got = faces(wenoz_folded, V)
    # f+ stencil of the face between cells 2 and 3 of a window
    assert np.allclose(got, 2.0 + 0.125 * (np.arange(6) + 2.5), rtol=1e-14)


def split_ref(D, d, u, v, w, c, g):
    t1, t2, t3, gm1 = 1.0 / (2.0 * g), 2.0 * (g - 1.0), (3.0 - g) / (2.0 * (g - 1.0)), g - 1.0
    vel = [u, v, w]
    un = vel[D]
    uc1, uc2 = un - c, un + c
    a = list(vel); b = list(vel)
    a[D], b[D] = uc1, uc2
    vvc1 = 0.5 * (a[0] * a[0] + a[1] * a[1] + a[2] * a[2])
    vvc2 = 0.5 * (b[0] * b[0] + b[1] * b[1] + b[2] * b[2])
    v2 = gm1 * (u * u + v * v + w * w)
    w2 = t3 * c * c
    E1, E2, E3 = un, un - c, un + c
    E1P, E2P, E3P = (E1 + np.abs(E1)) * 0.5, (E2 + np.abs(E2)) * 0.5, (E3 + np.abs(E3)) * 0.5
    E1M, E2M, E3M = E1 - E1P, E2 - E2P, E3 - E3P
    t0 = d * t1
    sp, sm = t2 * E1P + E2P + E3P, t2 * E1M + E2M + E3M
    fp = [t0 * sp]; fm = [t0 * sm]
    for m in range(3):
        if m == D:
            fp.append(t0 * (t2 * E1P * un + E2P * uc1 + E3P * uc2))
            fm.append(t0 * (t2 * E1M * un + E2M * uc1 + E3M * uc2))
        else:
            fp.append(t0 * vel[m] * sp)
            fm.append(t0 * vel[m] * sm)
    fp.append(t0 * (E1P * v2 + E2P * vvc1 + E3P * vvc2 + w2 * (E2P + E3P)))
    fm.append(t0 * (E1M * v2 + E2M * vvc1 + E3M * vvc2 + w2 * (E2M + E3M)))
    return np.array(fp), np.array(fm)


def split_grouped(D, d, u, v, w, c, g):
    t1, t2, t3, gm1 = 1.0 / (2.0 * g), 2.0 * (g - 1.0), (3.0 - g) / (2.0 * (g - 1.0)), g - 1.0
    vel = [u, v, w]
    un, ua, ub = vel[D], vel[(D + 1) % 3], vel[(D + 2) % 3]
    qt = ub * ub + ua * ua
    uc1, uc2 = un - c, un + c
    w2 = (t3 * c) * c
    v2 = gm1 * (un * un + qt)
    h1 = 0.5 * (uc1 * uc1 + qt) + w2
    h2 = 0.5 * (uc2 * uc2 + qt) + w2
    E1P, E2P, E3P = np.maximum(un, 0.0), np.maximum(uc1, 0.0), np.maximum(uc2, 0.0)
    E1M, E2M, E3M = np.minimum(un, 0.0), np.minimum(uc1, 0.0), np.minimum(uc2, 0.0)
    t0 = d * t1
    a1p, a1m = t2 * E1P, t2 * E1M
    rp, rm = t0 * ((a1p + E2P) + E3P), t0 * ((a1m + E2M) + E3M)
    fp = [rp]; fm = [rm]
    for m in range(3):
        if m == D:
            fp.append(t0 * (E3P * uc2 + (E2P * uc1 + a1p * un)))
            fm.append(t0 * (E3M * uc2 + (E2M * uc1 + a1m * un)))
        else:
            fp.append(rp * vel[m])
            fm.append(rm * vel[m])
    fp.append(t0 * (E3P * h2 + (E2P * h1 + E1P * v2)))
    fm.append(t0 * (E3M * h2 + (E2M * h1 + E1M * v2)))
    return np.array(fp), np.array(fm)


def test_split_grouped_matches_reference():
    rng = np.random.default_rng(7)
    n = 20000
    d = 10.0 ** rng.uniform(-3, 1, n)
    c = 10.0 ** rng.uniform(1, 3, n)
    u, v, w = (c * rng.uniform(-3, 3, n) for _ in range(3))
    u[:100] = 0.0                # exact zeros and sonic points among them
    v[100:200] = -c[100:200]
    for D in range(3):
        for g in (1.4, 1.29):
            rp, rm = split_ref(D, d, u, v, w, c, g)
            gp, gm = split_grouped(D, d, u, v, w, c, g)
            # per flux component against the magnitude of F+ and F- of that cell
            scale = np.maximum(np.abs(rp), np.abs(rm)).max(axis=0)
            assert (np.abs(gp - rp) / scale).max() < 4e-15   # measured: 5e-16
            assert (np.abs(gm - rm) / scale).max() < 4e-15
            # the eigenvalue parts are exact selects
            for x in (u, u - c, u + c):
                P = (x + np.abs(x)) * 0.5
                assert np.array_equal(P, np.maximum(x, 0.0)) and np.array_equal(x - P, np.minimum(x, 0.0))


def test_cfl_bound_from_largest_speed_is_exact():
    """min over cells of RN(dx / s) == RN(dx / max s), bit for bit."""
    rng = np.random.default_rng(11)
    for dx in (1.0 / 3.0, 0.1, 7.8125e-3, 1e-5 / 3.0):
        for _ in range(200):
            s = 10.0 ** rng.uniform(0, 4, 257) * (1.0 + rng.uniform(0, 1e-12, 257))
            assert np.min(dx / s) == dx / np.max(s)
        # neighbouring doubles
        s = np.nextafter(np.full(64, 340.0), np.inf) * (1.0 + np.arange(64) * 2.0 ** -52)
        assert np.min(dx / s) == dx / np.max(s)
