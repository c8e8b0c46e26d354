"""Chemistry surrogate pipeline on the GPU, at a small scale: samples from the
FP64 implicit substep, training on the tensor-core kernels, the guard with its
FP64 fallback, and the network embedded in the reacting level."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import ocfd
    return ocfd.Context()


@pytest.fixture(scope="module")
def trained(ctx):
    from ocfd import surrogate
    X, T = surrogate.generate(ctx, n_traj=8192, n_snap=96, seed=5)
    sur, rep = surrogate.train(ctx, X, T, epochs=30, batch=8192, lr=2e-3, seed=2)
    return X, T, sur, rep


def test_samples_are_physical(trained):
    import torch
    X, T, _, _ = trained
    assert X.shape[1] == 12 and T.shape[1] == 10 and X.shape[0] > 700000
    Y = X[:, 2:11]
    assert float(Y.min()) >= 0.0 and torch.allclose(Y.sum(1), torch.ones_like(Y[:, 0]), atol=1e-6)
    assert float(X[:, 0].min()) >= 250.0 and float(X[:, 0].max()) <= 3500.0
    # the FP64 substep conserves mass up to its clipping of negative partial
    # densities (large linearised steps clip): typically the increments of Y sum to ~0
    assert float(T[:, 1:].sum(1).abs().median()) < 1e-8


def test_training_lowers_the_loss(trained):
    _, _, _, rep = trained
    assert rep["final_train_loss"] < 0.7 * rep["first_epoch_loss"]
    assert rep["val_loss"] < 1.5 * rep["final_train_loss"] + 1e-3


def _timed(fn, reps=5):
    import torch
    fn()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def test_surrogate_substep_vs_fp64(ctx, trained):
    """What the network gains over the FP64 implicit substep it stands in for:
    the same substep of 1M 0D states (the reacting box's substep, 1.25 ns) at
    several times the cell rate, the guard's FP64 fallback keeping every state
    physical, and the temperature error within a small multiple of the
    temperature change itself (a broken network, wrong sign or scale, is off by
    orders of magnitude)."""
    import torch
    from ocfd import surrogate
    from ocfd.react import state_tpx
    _, _, sur, _ = trained
    rng = np.random.default_rng(9)
    n = 1 << 20
    Tm, p, X = surrogate.mixtures(rng, n)
    U0 = torch.as_tensor(state_tpx(ctx, Tm, p, X), device="cuda").contiguous()
    # advance so that radicals exist (0.4 us in steps of 10 ns: the linearised
    # implicit substep leaves the physical range on steps of 100 ns in a few
    # cells), keep the cells inside the tables' 250-3500 K
    for _ in range(40):
        surrogate.cells_advance(ctx, U0, dt=1e-8)
    T0 = surrogate.cells_props(ctx, U0)[0]
    keep = torch.isfinite(U0).all(0) & (T0 >= 250.0) & (T0 <= 3500.0)
    assert int(keep.sum()) > 0.99 * n
    U0 = U0[:, keep].contiguous()
    n = U0.shape[1]
    dt = 1.25e-9
    a, b = U0.clone(), U0.clone()
    surrogate.cells_advance(ctx, a, dt=dt)
    fb = surrogate.cells_surrogate(ctx, sur.net, sur.guard, b, dt)
    pa, pb, p0 = surrogate.cells_props(ctx, a), surrogate.cells_props(ctx, b), surrogate.cells_props(ctx, U0)
    assert 0 <= fb < n // 20
    assert torch.isfinite(b).all() and float(b[5:].min()) >= 0.0
    dT_true = float((pa[0] - p0[0]).abs().mean())
    err = float((pb[0] - pa[0]).abs().mean())
    assert err < 3.0 * dT_true, (err, dT_true)
    # density and momentum are untouched; accepted increments conserve the
    # elements, so the species mass is unchanged but for the clip of partial
    # densities driven below zero (the guard admits Y + dY >= -y_tol)
    assert torch.equal(b[:4], U0[:4])
    dm = (b[5:].sum(0) - U0[5:].sum(0)).abs() / b[0]
    assert float(dm.median()) < 1e-6 and float(dm.max()) < 2e-3
    Ua, Ub = U0.clone(), U0.clone()
    t_fp64 = _timed(lambda: surrogate.cells_advance(ctx, Ua, dt=dt))
    t_sur = _timed(lambda: surrogate.cells_surrogate(ctx, sur.net, sur.guard, Ub, dt))
    assert t_sur * 3.0 < t_fp64, (t_sur, t_fp64)


def test_reacting_level_with_surrogate(ctx, trained):
    from ocfd.cases import react_cube
    from ocfd.level import chop_domain
    from ocfd.react import Reactor
    from ocfd import surrogate
    import ctypes
    _, _, sur, _ = trained
    case = react_cube(ctx, n=32, length=0.01 * 32 / 128, seed=7)
    boxes = chop_domain(case["n"], 16)
    out = {}
    for mode in ("plain", "surrogate"):
        R = Reactor(ctx, boxes, (31, 31, 31), case["dx"], dt=1e-8, rk_order=2, chem_substeps=4)
        R.level.set_global(case["G"])
        if mode == "surrogate":
            from ocfd._abi import check, load
            check(load().ocfd_react_set_surrogate(R.h, sur.net.h, ctypes.byref(sur.guard)), "set_surrogate")
        R.advance(3)
        out[mode] = R.level.get_global()
        if mode == "surrogate":
            fb = ctypes.c_int64()
            check(load().ocfd_react_fallbacks(R.h, ctypes.byref(fb), None), "fallbacks")
            out["fb"] = fb.value
        R.close()
    a, b = out["plain"], out["surrogate"]
    assert np.isfinite(b).all() and b[5:].min() >= 0.0
    # the network serves most cells (3 steps x 8 substeps of 32^3 cells): the
    # box's states lie inside the guard's training ranges
    assert 0 <= out["fb"] < 0.5 * 3 * 8 * 32 ** 3
    # density is untouched by chemistry; the temperature stays close to the FP64
    # run (the induction-phase radicals and products of a 30 ns run are 1e-14 in
    # mass fraction, below the network's absolute error: their errors are
    # reported by the benchmark, not bounded here)
    assert np.abs(b[0] - a[0]).max() / a[0].max() < 1e-4
    import torch
    props = lambda U: surrogate.cells_props(ctx, torch.as_tensor(U.reshape(14, -1), device="cuda").contiguous())
    Ta, Tb = props(a)[0], props(b)[0]
    assert float((Tb - Ta).abs().sum() / Ta.abs().sum()) < 5e-3


def _advanced_states(ctx, n, seed, steps=40):
    """0D H2/air states advanced at constant volume for steps x 10 ns (radicals
    present), inside the tables' 250-3500 K"""
    import torch
    from ocfd import surrogate
    from ocfd.react import state_tpx
    rng = np.random.default_rng(seed)
    Tm, p, X = surrogate.mixtures(rng, n)
    U = torch.as_tensor(state_tpx(ctx, Tm, p, X), device="cuda").contiguous()
    for _ in range(steps):
        surrogate.cells_advance(ctx, U, dt=1e-8)
    T0 = surrogate.cells_props(ctx, U)[0]
    keep = torch.isfinite(U).all(0) & (T0 >= 250.0) & (T0 <= 3500.0)
    return U[:, keep].contiguous()


def test_isobaric_restoration(ctx):
    """After a constant-volume substep the isobaric restoration brings each cell
    back to its pressure at the enthalpy e + p0 / rho (rho before the
    restoration), keeps the mass fractions, and leaves a cell already at p0
    unchanged."""
    import torch
    from ocfd import surrogate
    U = _advanced_states(ctx, 4096, seed=11, steps=5)
    n = U.shape[1]
    p0 = surrogate.cells_props(ctx, U)[1].contiguous()
    # a cell already at its pressure: unchanged
    V = U.clone()
    surrogate.cells_isobaric(ctx, V, p0)
    assert float(((V - U).abs().amax(1) / U.abs().amax(1).clamp_min(1e-300)).max()) < 1e-9
    # one constant-volume substep raises p in the igniting cells; restore
    surrogate.cells_advance(ctx, U, dt=1e-7)
    pr = surrogate.cells_props(ctx, U)
    h_target = U[4] / U[0] + p0 / U[0]
    W = U.clone()
    surrogate.cells_isobaric(ctx, W, p0)
    pw = surrogate.cells_props(ctx, W)
    assert float(((pr[1] - p0).abs() / p0).max()) > 1e-3      # the substep moved p
    assert float(((pw[1] - p0).abs() / p0).max()) < 1e-9
    h = W[4] / W[0] + pw[1] / W[0]
    assert float(((h - h_target).abs() / h_target.abs().clamp_min(1e3)).max()) < 1e-9
    assert float((pw[2:] - pr[2:]).abs().max()) < 1e-12
    assert torch.equal(W[1:4], torch.zeros_like(W[1:4]))
    assert n > 4000


def test_constant_pressure_generator(ctx):
    """mode="pressure" samples every snapshot of a trajectory at its initial
    pressure"""
    import torch
    from ocfd import surrogate
    n_traj, n_snap = 512, 6
    X, T = surrogate.generate(ctx, n_traj=n_traj, n_snap=n_snap, seed=3, mode="pressure")
    assert X.shape[0] == n_traj * n_snap
    _, p0, _ = surrogate.mixtures(np.random.default_rng(3), n_traj)
    p = X[:, 1].double().cpu().numpy().reshape(n_snap, n_traj)
    assert np.abs(p / p0[None] - 1.0).max() < 1e-6          # float32 features
    # the trajectories evolved: some cells ignite (T rises at constant p)
    Tf = X[:, 0].double().cpu().numpy().reshape(n_snap, n_traj)
    assert (Tf[-1] - Tf[0]).max() > 10.0
    with pytest.raises(ValueError):
        surrogate.generate(ctx, n_traj=8, n_snap=1, mode="enthalpy")


def test_per_output_guard_is_monotone(ctx, trained):
    """Tightening the per-output criterion sends a growing share of cells to the
    FP64 substep and brings the species error down toward it."""
    import torch
    from ocfd import surrogate
    _, _, sur, _ = trained
    U0 = _advanced_states(ctx, 1 << 18, seed=21)
    dt = 1.25e-9
    ref = U0.clone()
    surrogate.cells_advance(ctx, ref, dt=dt)
    pr = surrogate.cells_props(ctx, ref)
    fbs, errs = [], []
    for d in (0.0, 1.0, 0.1, 0.01, 0.001):
        g = sur.guard.with_dy_rel(d)
        b = U0.clone()
        fbs.append(surrogate.cells_surrogate(ctx, sur.net, g, b, dt))
        pb = surrogate.cells_props(ctx, b)
        errs.append(float((pb[2 + 5] - pr[2 + 5]).abs().sum() / pr[2 + 5].abs().sum()))
    assert all(a <= b for a, b in zip(fbs, fbs[1:])), fbs
    assert fbs[-1] > fbs[0]
    assert errs[-1] <= errs[0] + 1e-12, errs
    # the struct passed through the C ABI carries the two new fields
    g = sur.guard.with_dy_rel(0.5, 1e-5)
    h = surrogate.Guard.from_buffer_copy(g)
    assert (h.dy_rel_max, h.y_floor, h.elem_tol) == (0.5, 1e-5, sur.guard.elem_tol)
