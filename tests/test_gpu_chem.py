"""Chemistry substep and species renormalisation on the GPU against the oracle
and the reference's golden fixture.  exp/log/pow differ between CUDA and the
host libm by a few ulps, so the tolerance is 1e-11 relative (norm-wise per
quantity) for one substep."""
import numpy as np
import pytest

import inputs
from conftest import golden

pytestmark = pytest.mark.gpu


def relerr(a, b):
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / (den if den > 0 else 1.0))


@pytest.fixture(scope="module")
def ctx():
    import ocfd
    return ocfd.Context()


def run_chem(ctx, S, sp, dt, nsub=1):
    import torch
    n = S.shape[1]
    St = torch.from_numpy(np.ascontiguousarray(S)).reshape(5, 1, 1, n).cuda()
    Rt = torch.from_numpy(np.ascontiguousarray(sp)).reshape(9, 1, 1, n).cuda()
    for _ in range(nsub):
        ctx.chem_advance_box(St, Rt, (0, 0, 0), (n - 1, 0, 0), dt)
    torch.cuda.synchronize()
    return St.reshape(5, n).cpu().numpy(), Rt.reshape(9, n).cpu().numpy()


def test_chem_vs_golden(ctx):
    g = golden("chem_advance")
    S, sp = run_chem(ctx, g["S"], g["spec"], float(g["dt"]), int(g["nsub"]))
    assert relerr(S[4], g["S_out"][4]) < 1e-11
    for n in range(9):
        assert relerr(sp[n], g["spec_out"][n]) < 1e-11 or np.abs(sp[n] - g["spec_out"][n]).max() < 1e-14


@pytest.mark.parametrize("dt", [1e-8, 3e-7, 1e-5])
def test_chem_vs_oracle(ctx, oracle, dt):
    S, sp = inputs.chem_state(10, 8, 6, seed=77, oracle=oracle)   # 18*16*14 cells incl. ghosts
    S = np.ascontiguousarray(S.reshape(5, -1)); sp = np.ascontiguousarray(sp.reshape(9, -1))
    So, spo = S.copy(), sp.copy()
    oracle.chem_advance(So, spo, dt)
    Sg, spg = run_chem(ctx, S, sp, dt)
    assert np.isfinite(Sg).all() and np.isfinite(spg).all()
    assert relerr(Sg[4], So[4]) < 1e-11
    tot = np.abs(spo).max()
    assert np.abs(spg - spo).max() / tot < 1e-11


def test_chem_ignition_trajectory(ctx, oracle):
    """400 substeps of 1e-7 s of a stoichiometric H2/air cell at 1400 K (it
    ignites after about 20 us): the GPU and CPU integrators follow the same
    trajectory to the burnt state (temperature within 1e-8 relative)."""
    X = np.zeros(9); X[0] = 0.2958; X[1] = 0.1479; X[8] = 0.5563
    Y = oracle.ckxty(X)
    rho = oracle.ckrhoy(101325.0, 1400.0, Y)
    r = rho * Y
    E = oracle.ckubms(1400.0, r)
    S = np.array([[rho], [0.0], [0.0], [0.0], [E]]); sp = r.reshape(9, 1).copy()
    So, spo = S.copy(), sp.copy()
    import torch
    St = torch.from_numpy(S.copy()).reshape(5, 1, 1, 1).cuda()
    Rt = torch.from_numpy(sp.copy()).reshape(9, 1, 1, 1).cuda()
    for _ in range(400):
        oracle.chem_advance(So, spo, 1e-7)
        ctx.chem_advance_box(St, Rt, (0, 0, 0), (0, 0, 0), 1e-7)
    Sg = St.reshape(5, 1).cpu().numpy(); spg = Rt.reshape(9, 1).cpu().numpy()
    Tg = oracle.get_t_given_ey(Sg[4, 0], spg[:, 0]); To = oracle.get_t_given_ey(So[4, 0], spo[:, 0])
    assert To > 2000.0   # ignited
    assert abs(Tg - To) / To < 1e-8


def test_spec_renorm_vs_oracle(ctx, oracle):
    import torch
    S, sp = inputs.chem_state(6, 5, 4, seed=78, oracle=oracle)
    S = np.ascontiguousarray(S.reshape(5, -1)); sp = np.ascontiguousarray(sp.reshape(9, -1))
    sp[2] -= 0.1 * sp[2].max()      # some negative partial densities
    S[0] *= 1.01
    So, spo = S.copy(), sp.copy()
    oracle.spec_renorm(So, spo)
    n = S.shape[1]
    St = torch.from_numpy(S).reshape(5, 1, 1, n).cuda()
    Rt = torch.from_numpy(sp.copy()).reshape(9, 1, 1, n).cuda()
    ctx.spec_renorm_box(St, Rt, (0, 0, 0), (n - 1, 0, 0))
    assert np.array_equal(Rt.reshape(9, n).cpu().numpy(), spo)
