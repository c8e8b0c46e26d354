"""include/ocfd/compat.H: the reference's per-point functions (c2prim,
flux_split_x/y/z, reconstruction_x/y/z, compute_visc_x/y/z, divop) under their
own names, computed by this library's point arithmetic.  tests/compat_chain.cu
chains them in the loop order of Source/Advance.cpp:245-329; compiled for the
host with nvcc, the chain's dS/dt must equal the oracle's regular-box RHS (which
is pinned bit for bit to the reference's own kernel headers) - exactly where
neither build contracts multiply-adds (x86-64 baseline), to 1e-14 otherwise."""
import ctypes
import os
import platform
import subprocess

import numpy as np
import pytest

import inputs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")


@pytest.fixture(scope="module")
def chain(tmp_path_factory):
    if not os.path.exists(NVCC):
        pytest.skip("nvcc not present")
    out = str(tmp_path_factory.mktemp("compat") / "libcompat.so")
    cmd = [NVCC, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2", "-Xcompiler", "-fPIC",
           "-shared", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "opencfd-amr_gb300", "csrc"),
           os.path.join(ROOT, "tests", "compat_chain.cu"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(out)
    lib.compat_rhs_regular.restype = ctypes.c_int
    return lib


def run_chain(lib, S, dxinv, visc):
    from ocfd.context import default_parm
    _, gz, gy, gx = S.shape
    nx, ny, nz = gx - 8, gy - 8, gz - 8
    S = np.ascontiguousarray(S)
    out = np.full((5, nz, ny, nx), np.nan)
    dx = (ctypes.c_double * 3)(*dxinv)
    p = default_parm()
    lib.compat_rhs_regular(S.ctypes.data_as(ctypes.c_void_p), nx, ny, nz, dx, int(visc), ctypes.byref(p),
                           out.ctypes.data_as(ctypes.c_void_p))
    return out


@pytest.mark.parametrize("shape,seed", [((9, 7, 5), 1), ((12, 6, 4), 2), ((5, 11, 6), 3)])
@pytest.mark.parametrize("visc", [False, True])
def test_compat_chain_equals_oracle(chain, oracle, shape, seed, visc):
    S = inputs.ideal_state(*shape, seed)
    dxinv = [11.0, 9.0, 7.0]
    if visc:   # dimensional air-like state so the viscous terms matter
        S = S.copy(); S[0] *= 1.2; S[1:4] *= 360.0; S[4] *= 1.0e5
        dxinv = [1.0e4, 1.2e4, 0.9e4]
    ref, _ = oracle.rhs_regular(S, dxinv, do_visc=visc)
    got = run_chain(chain, S, dxinv, visc)
    assert np.isfinite(got).all()
    if platform.machine() in ("x86_64", "AMD64"):
        assert np.array_equal(got, ref)
    else:
        assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max()
