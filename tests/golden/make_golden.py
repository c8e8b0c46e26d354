"""Generate tests/golden/*.npz from OpenCFD-AMR's own kernels.

Run here, where the reference tree exists:
    make -C oracle ref && python tests/golden/make_golden.py
It compiles nothing itself; it calls oracle/_ref (the reference kernel headers
and Source/Constants.cpp compiled unmodified against the project's AMReX
stand-ins) on small seeded inputs and stores inputs and outputs.  The fixtures
then pin the CPU oracle and the CUDA kernels on machines without the reference.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
sys.path.insert(0, os.path.join(HERE, ".."))

from oracle import Oracle, RefOracle, build_ref  # noqa: E402
import inputs  # noqa: E402


def main():
    build_ref()
    ref = RefOracle()
    o = Oracle()  # only used to build chemistry states (energy from CKUBMS)
    out = {}

    # regular box, nondimensional shock-tube-like state
    S = inputs.ideal_state(6, 5, 4, seed=101)
    dxinv = np.array([11.0, 12.0, 13.0])
    dS, f = ref.rhs_regular(S, dxinv, do_visc=False)
    out["regular_inviscid"] = dict(S=S, dxinv=dxinv, dSdt=dS, fx=f[0], fy=f[1], fz=f[2])

    # regular box, dimensional air state for the viscous terms
    S = inputs.ideal_state(6, 5, 4, seed=102)
    S[0] *= 1.2; S[1:4] *= 1.2 * 300.0; S[4] = S[4] * 1.0e5 + (1.2 * 300.0 ** 2 - 1.0) * S[4]
    dxinv = np.array([1.0e4, 1.1e4, 0.9e4])
    dS, f = ref.rhs_regular(S, dxinv, do_visc=True)
    out["regular_viscous"] = dict(S=S, dxinv=dxinv, dSdt=dS, fx=f[0], fy=f[1], fz=f[2])

    # cut-cell box
    S = inputs.ideal_state(8, 8, 3, seed=103)
    g = inputs.cylinder_box(8, 8, 3)
    dxinv = np.array([3.0, 3.0, 3.0])
    for visc in (0, 1):
        for red in (0, 1):
            dS, f = ref.rhs_eb(S, g, dxinv, visc, red)
            out[f"eb_v{visc}_r{red}"] = dict(S=S, dxinv=dxinv, dSdt=dS, fx=f[0], fy=f[1], fz=f[2],
                                             **{k: v for k, v in g.items()})

    # multispecies boxes
    S, sp = inputs.chem_state(4, 4, 3, seed=104, oracle=o)
    dxinv = np.array([1.0e4, 1.0e4, 1.0e4])
    dS, dSs, f, fs, fd = ref.rhs_chem(S, sp, dxinv, do_visc=True)
    out["chem_regular"] = dict(S=S, spec=sp, dxinv=dxinv, dSdt=dS, dSdt_spec=dSs,
                               fx=f[0], fy=f[1], fz=f[2], fxs=fs[0], fys=fs[1], fzs=fs[2],
                               fxd=fd[0], fyd=fd[1], fzd=fd[2])
    g = inputs.cylinder_box(4, 4, 3)
    dS, dSs, f, fs, fd = ref.rhs_chem(S, sp, dxinv, do_visc=True, geom=g)
    out["chem_eb"] = dict(S=S, spec=sp, dxinv=dxinv, dSdt=dS, dSdt_spec=dSs,
                          fx=f[0], fy=f[1], fz=f[2], fxs=fs[0], fys=fs[1], fzs=fs[2],
                          **{k: v for k, v in g.items()})
    mu, lam, D = ref.transport(S, sp)
    out["transport"] = dict(S=S, spec=sp, mu=mu, lam=lam, D=D)
    q = ref.c2prim(S, sp)
    out["c2prim_chem"] = dict(S=S, spec=sp, q=q)

    # chemistry substeps on 300 cells of the same state
    S2 = np.ascontiguousarray(S.reshape(5, -1)[:, :300])
    s2 = np.ascontiguousarray(sp.reshape(9, -1)[:, :300])
    S_out, s_out = S2.copy(), s2.copy()
    for _ in range(2):
        ref.chem_advance(S_out, s_out, 1.0e-7)
    out["chem_advance"] = dict(S=S2, spec=s2, dt=np.array(1.0e-7), nsub=np.array(2),
                               S_out=S_out, spec_out=s_out)

    # CFL bound
    S = inputs.ideal_state(6, 5, 4, seed=105)
    out["estdt"] = dict(S=S, dx=np.array([0.1, 0.11, 0.09]),
                        dt=np.array(ref.estdt(S, [0.1, 0.11, 0.09])))

    for name, d in out.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print("wrote", name)


if __name__ == "__main__":
    main()
