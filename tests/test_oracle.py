"""The CPU oracle, pinned against the reference.

* golden pair: the jet inflow constants hard-coded in Exec/7_JET/prob.cpp:18-28
  are what Test/chemical_test.cpp computes; the oracle must reproduce them;
* golden fixtures (tests/golden, produced by the reference's own kernels);
* where the reference tree exists: bit-for-bit against oracle/_ref on fresh
  seeds, and the reference's standalone chemistry program.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import golden, ROOT
import inputs


def relerr(a, b):
    a = np.asarray(a); b = np.asarray(b)
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / (den if den > 0 else 1.0))


def test_parm_defaults(oracle):
    p = oracle.parm
    assert p.eos_gamma == 1.4 and p.Rg == p.Ru / p.eos_m
    assert p.kOverMu == p.cp / p.Pr


def test_jet_golden_pair(oracle):
    # Exec/7_JET/prob.cpp:18-22 inner (jet) state at 305 K, X_H2=0.15, X_N2=0.85
    X = np.zeros(9); X[0] = 0.15; X[8] = 0.85
    Y = oracle.ckxty(X)
    rho = oracle.ckrhoy(101325.0, 305.0, Y)
    e = oracle.ckubms(305.0, rho * Y)
    assert rho == pytest.approx(0.963512265437802995, rel=1e-15)
    assert e == pytest.approx(245428.076382951345, rel=1e-15)
    # Exec/7_JET/prob.cpp:24-28,36-37 outer state at 1150 K, X_O2=0.21, X_N2=0.79
    X = np.zeros(9); X[1] = 0.21; X[8] = 0.79
    Y = oracle.ckxty(X)
    rho = oracle.ckrhoy(101325.0, 1150.0, Y)
    assert rho == pytest.approx(0.305731395505996983, rel=1e-15)
    assert oracle.ckubms(1150.0, rho * Y) == pytest.approx(271976.980564150028, rel=1e-15)
    assert Y[1] == pytest.approx(0.232909, abs=5e-7)
    # temperature inversion recovers T (Newton tolerance 1e-7 K, LiDryer.H:838)
    assert oracle.get_t_given_ey(oracle.ckubms(1150.0, rho * Y), rho * Y) == pytest.approx(1150.0, abs=1e-6)


def test_temperature_inversion_roundtrip(oracle):
    rng = np.random.default_rng(5)
    for T in rng.uniform(300, 3000, 20):
        X = rng.dirichlet(np.ones(9))
        Y = oracle.ckxty(X)
        rho = oracle.ckrhoy(101325.0, T, Y)
        e = oracle.ckubms(T, rho * Y)
        assert oracle.get_t_given_ey(e, rho * Y) == pytest.approx(T, rel=1e-9)


@pytest.mark.parametrize("name", ["regular_inviscid", "regular_viscous"])
def test_oracle_regular_vs_golden(oracle, name):
    g = golden(name)
    dS, f = oracle.rhs_regular(g["S"], g["dxinv"], do_visc=name.endswith("viscous"))
    assert np.array_equal(dS, g["dSdt"])
    for a, k in zip(f, ("fx", "fy", "fz")):
        assert np.array_equal(a, g[k])


@pytest.mark.parametrize("visc,red", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_oracle_eb_vs_golden(oracle, visc, red):
    g = golden(f"eb_v{visc}_r{red}")
    dS, f = oracle.rhs_eb(g["S"], g, g["dxinv"], visc, red)
    assert np.array_equal(dS, g["dSdt"])
    for a, k in zip(f, ("fx", "fy", "fz")):
        assert np.array_equal(a, g[k])


# exp/log/pow come from the platform's libm: allow a few ulps between machines
CHEM_RTOL = 1e-13


def test_oracle_chem_vs_golden(oracle):
    g = golden("chem_regular")
    dS, dSs, f, fs, fd = oracle.rhs_chem(g["S"], g["spec"], g["dxinv"], do_visc=True)
    assert relerr(dS, g["dSdt"]) < CHEM_RTOL
    assert relerr(dSs, g["dSdt_spec"]) < CHEM_RTOL
    for a, k in zip(fd, ("fxd", "fyd", "fzd")):
        assert relerr(a, g[k]) < CHEM_RTOL
    g = golden("chem_eb")
    geom = {k: g[k] for k in ("flag", "vfrac", "apx", "apy", "apz")}
    dS, dSs, f, fs, fd = oracle.rhs_chem(g["S"], g["spec"], g["dxinv"], do_visc=True, geom=geom)
    assert np.array_equal(dS, g["dSdt"])   # the reference leaves the flow dSdt zero in cut CHEM boxes
    assert relerr(dSs, g["dSdt_spec"]) < CHEM_RTOL


def test_oracle_transport_c2prim_vs_golden(oracle):
    g = golden("transport")
    mu, lam, D = oracle.transport(g["S"], g["spec"])
    assert relerr(mu, g["mu"]) < CHEM_RTOL and relerr(lam, g["lam"]) < CHEM_RTOL
    assert relerr(D, g["D"]) < CHEM_RTOL
    g = golden("c2prim_chem")
    q = oracle.c2prim(g["S"], g["spec"])
    for n in range(8):
        assert relerr(q[n], g["q"][n]) < CHEM_RTOL


def test_oracle_chem_advance_vs_golden(oracle):
    g = golden("chem_advance")
    S, sp = g["S"].copy(), g["spec"].copy()
    for _ in range(int(g["nsub"])):
        oracle.chem_advance(S, sp, float(g["dt"]))
    assert relerr(S, g["S_out"]) < 1e-12
    assert relerr(sp, g["spec_out"]) < 1e-12


def test_oracle_estdt_vs_golden(oracle):
    g = golden("estdt")
    assert oracle.estdt(g["S"], g["dx"]) == float(g["dt"])


# ---------------------------------------------------------------- vs reference
def test_tables_match_reference(oracle, ref):
    t = ref.chem_tables()
    p = oracle.parm
    assert np.array_equal(np.array(p.mw), t["mw"])
    assert np.array_equal(np.array(p.nasa_lo), t["lo"]) and np.array_equal(np.array(p.nasa_hi), t["hi"])
    assert np.array_equal(np.array(p.HP), t["HP"]) and np.array_equal(np.array(p.A0), t["A0"])
    assert np.array_equal(np.array(p.visccoeff), t["visc"])
    assert np.array_equal(np.array(p.conductcoeff), t["cond"])
    assert np.array_equal(np.array(p.diffcoeff), t["diff"])
    assert ref.parm_scalars() == [getattr(p, f) for f, _ in p._fields_[:16]]


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_bitexact_vs_reference(oracle, ref, seed):
    S = inputs.ideal_state(9, 7, 5, seed)
    for visc in (0, 1):
        a, fa = oracle.rhs_regular(S, [11.0, 9.0, 7.0], visc)
        b, fb = ref.rhs_regular(S, [11.0, 9.0, 7.0], visc)
        assert np.array_equal(a, b)
    g = inputs.cylinder_box(9, 7, 5)
    for visc in (0, 1):
        a, _ = oracle.rhs_eb(S, g, [3.0, 3.0, 3.0], visc, 1)
        b, _ = ref.rhs_eb(S, g, [3.0, 3.0, 3.0], visc, 1)
        assert np.array_equal(a, b)
    Sc, sp = inputs.chem_state(5, 4, 3, seed, oracle)
    for visc in (0, 1):
        a = oracle.rhs_chem(Sc, sp, [1e4, 1e4, 1e4], visc)
        b = ref.rhs_chem(Sc, sp, [1e4, 1e4, 1e4], visc)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    S2 = np.ascontiguousarray(Sc.reshape(5, -1)[:, :200]); s2 = np.ascontiguousarray(sp.reshape(9, -1)[:, :200])
    S3, s3 = S2.copy(), s2.copy()
    oracle.chem_advance(S2, s2, 3e-7); ref.chem_advance(S3, s3, 3e-7)
    assert np.array_equal(S2, S3) and np.array_equal(s2, s3)


def test_point_thermo_vs_reference(oracle, ref):
    rng = np.random.default_rng(9)
    for _ in range(10):
        T = rng.uniform(280, 3200)
        X = rng.dirichlet(np.ones(9))
        c = rng.uniform(0, 1e-6, 9)
        assert np.array_equal(oracle.production_rate(c, T)[0], ref.production_rate(c, T)[0])
        assert np.array_equal(oracle.production_rate(c, T)[1], ref.production_rate(c, T)[1])
        assert oracle.mixture_properties(T, X) == ref.mixture_properties(T, X)
        assert np.array_equal(oracle.mix_diff_coeffs(T, 1e5, X), ref.mix_diff_coeffs(T, 1e5, X))
        assert np.array_equal(oracle.species_enthalpy(T), ref.species_enthalpy(T))
        A = rng.standard_normal((9, 9)) + 5 * np.eye(9); b = rng.standard_normal(9)
        assert np.array_equal(oracle.gauss(A, b), ref.gauss(A, b))


def test_reference_chemical_test_program(tmp_path):
    exe = os.path.join(ROOT, "oracle", "_ref", "chemical_test")
    if not os.path.exists(exe):
        pytest.skip("reference programs not built on this machine")
    out = subprocess.run([exe], capture_output=True, text=True, cwd=str(tmp_path)).stdout
    assert "rho = 0.963512265437802995" in out
    assert "E = 245428.076382951345" in out


def test_reference_flop_counts():
    """Operation counts of the reference's ideal-gas point functions, from its
    own headers compiled with a counting Real (make -C oracle flops); these are
    the algorithmic FLOPs per cell-stage quoted for the roofline."""
    import json
    from oracle import reference_dir
    ref = reference_dir()
    if ref is None:
        pytest.skip("reference sources not present on this machine")
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "flops", "REF=" + ref],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "flop_count")], capture_output=True, text=True)
    c = json.loads(out.stdout)
    flops = {k: v["add"] + v["mul"] + v["div"] + v["sqrt"] for k, v in c.items()}
    assert flops["c2prim"] == 19 and c["c2prim"]["div"] == 2 and c["c2prim"]["sqrt"] == 1
    for d in "xyz":
        assert flops["flux_split_" + d] == 103
        assert flops["reconstruction_" + d] == 191 and c["reconstruction_" + d]["div"] == 14
        assert flops["compute_visc_" + d] == 68
    assert flops["divop"] == 8
    per_cell = flops["c2prim"] + sum(flops["flux_split_" + d] + 5 * flops["reconstruction_" + d] for d in "xyz") \
        + 5 * flops["divop"]
    assert per_cell == 3233
    out = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "flop_count_chem")], capture_output=True, text=True)
    c = json.loads(out.stdout)
    step = c["chemical_advance_cell"]
    # one implicit substep of an H2/air cell at 1500 K: ~9.9 k FLOPs, ~1000 of them
    # divisions, 47 exp / log / pow
    assert step["add"] + step["mul"] + step["div"] == 9869 and step["div"] == 995 and step["other"] == 47
    # the viscous multispecies RHS of one cell (Source/CHEM/FlowAdvance.cpp:157-403):
    # c2prim_rgas and transport once, per direction the splits, 14 components'
    # WENO-Z, the diffusive and viscous fluxes, then divop on 14 components
    f = {k: v["add"] + v["mul"] + v["div"] + v["sqrt"] for k, v in c.items()}
    per_dir = f["flux_split_x_chem"] + f["species_split_x"] + 14 * f["reconstruction_x_chem"] + f["diffusion_x"] \
        + f["compute_visc_x_multi"]
    assert f["c2prim_rgas"] + f["transport_cell"] + 3 * per_dir + 14 * 8 == 13708
