"""The allocation-free cut-cell RHS entry point, through the C ABI.

ocfd_rhs_eb_box_f64_static_scratch serves callers that cannot let a library
allocate device memory (an application that owns all device memory through its
own pool, or code where a cudaMalloc, which can synchronise the device, must
not happen).  It must give the same results as ocfd_rhs_eb_box_f64 (the
ordinary entry point, which takes its scratch from the context pool), on two
calls in a row - the second call reuses the shared static scratch the first
one left behind - and it must refuse a box larger than its fixed scratch.

This file is named so that pytest collects it last; it creates its own
context, so it also passes when run alone in a fresh process.  One test runs in
a child process of its own, where nothing else has touched the library: after
the context exists, the first call must not change the device's free memory
(the static array and the call's device code are made resident when the
context is created, not lazily by the first call).
"""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

import inputs

pytestmark = pytest.mark.gpu
TOL = 1e-12   # the tolerance of the other EB parity tests


def relerr(a, b):
    groups = [(0,), (1, 2, 3), (4,)]
    e = 0.0
    for g in groups:
        den = max(np.abs(b[list(g)]).max(), 1e-300)
        e = max(e, float(np.abs(a[list(g)] - b[list(g)]).max() / den))
    return e


@pytest.fixture(scope="module")
def api():
    import ocfd
    from ocfd._abi import Array4, Box, Flag4, declare
    argtypes = [ctypes.c_void_p, ctypes.POINTER(Array4), ctypes.POINTER(Array4), ctypes.POINTER(Array4),
                ctypes.POINTER(Flag4), ctypes.POINTER(Array4), ctypes.POINTER(Array4),
                ctypes.POINTER(Array4), ctypes.POINTER(Array4), ctypes.c_void_p, ctypes.POINTER(Array4),
                Box, ctypes.POINTER(ctypes.c_double), ctypes.c_uint, ctypes.c_void_p]
    declare("ocfd_rhs_eb_box_f64_static_scratch", ctypes.c_int, argtypes)
    ctx = ocfd.Context()
    return ocfd, ctx


def call(api, name, S, geom, lo, dxinv, flags, with_flux):
    """Run entry point `name` on host arrays; returns (dSdt, face fluxes or None)."""
    import torch
    ocfd, ctx = api
    L = ocfd.load()
    _, gz, gy, gx = S.shape
    nx, ny, nz = gx - 8, gy - 8, gz - 8
    hi = (lo[0] + nx - 1, lo[1] + ny - 1, lo[2] + nz - 1)
    g4 = tuple(x - 4 for x in lo)
    St = torch.from_numpy(np.ascontiguousarray(S)).cuda()
    dS = torch.full((5, nz, ny, nx), float("nan"), dtype=torch.float64, device="cuda")
    dev = {k: torch.from_numpy(np.ascontiguousarray(geom[k])).cuda() for k in ("vfrac", "apx", "apy", "apz")}
    dev["flag"] = torch.from_numpy(np.ascontiguousarray(geom["flag"]).view(np.int32)).cuda()
    fl, fl_arr = None, None
    if with_flux:
        fl = [torch.full((5, nz + (d == 2), ny + (d == 1), nx + (d == 0)), float("nan"),
                         dtype=torch.float64, device="cuda") for d in range(3)]
        fl_arr = (ocfd.Array4 * 3)(*[ocfd.array4(f, lo) for f in fl])
    aS, aD = ocfd.array4(St, g4), ocfd.array4(dS, lo)
    af, av = ocfd.flag4(dev["flag"], g4), ocfd.array4(dev["vfrac"], g4)
    ap = [ocfd.array4(dev[k], lo) for k in ("apx", "apy", "apz")]
    dx = (ctypes.c_double * 3)(*dxinv)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = getattr(L, name)(ctx.h, ctypes.byref(aS), ctypes.byref(aD), fl_arr, ctypes.byref(af),
                          ctypes.byref(av), ctypes.byref(ap[0]), ctypes.byref(ap[1]),
                          ctypes.byref(ap[2]), None, None, ocfd.box(lo, hi), dx, flags, stream)
    ocfd.check(st, name)
    torch.cuda.synchronize()
    return dS.cpu().numpy(), ([f.cpu().numpy() for f in fl] if fl else None)


@pytest.mark.parametrize("with_flux", [False, True])
def test_static_scratch_matches_pooled_entry_point_twice(api, with_flux):
    cases = [((20, 18, 6), (8, -4, 2), 41, 1),      # viscous
             ((14, 22, 5), (-6, 30, 0), 42, 2)]     # redistribution, different box shape
    for shape, lo, seed, flags in cases:           # two calls in a row on the shared scratch
        S = inputs.ideal_state(*shape, seed)
        geom = inputs.cylinder_box(*shape)
        ref, rf = call(api, "ocfd_rhs_eb_box_f64", S, geom, lo, [4.0, 4.0, 4.0], flags, with_flux)
        got, gf = call(api, "ocfd_rhs_eb_box_f64_static_scratch", S, geom, lo, [4.0, 4.0, 4.0], flags,
                       with_flux)
        assert np.isfinite(got).all()
        assert relerr(got, ref) <= TOL
        if with_flux:
            for d in range(3):
                assert relerr(gf[d], rf[d]) <= TOL


def test_static_scratch_rejects_oversized_box(api):
    ocfd, _ = api
    shape = (80, 80, 40)   # 7 * 84 * 84 * 44 doubles > the 2^21-double static scratch
    S = np.zeros((5, shape[2] + 8, shape[1] + 8, shape[0] + 8))
    S[0] = 1.0; S[4] = 2.5
    geom = inputs.cylinder_box(*shape)
    with pytest.raises(ocfd.OcfdError) as e:
        call(api, "ocfd_rhs_eb_box_f64_static_scratch", S, geom, (0, 0, 0), [1.0, 1.0, 1.0], 0, True)
    assert e.value.status == 1 and "static scratch" in str(e.value)


_FRESH = r"""
import ctypes, sys
sys.path[:0] = [{paths}]
import numpy as np, torch
import ocfd, inputs
from ocfd._abi import Array4, Box, Flag4, declare
argtypes = [ctypes.c_void_p, ctypes.POINTER(Array4), ctypes.POINTER(Array4), ctypes.POINTER(Array4),
            ctypes.POINTER(Flag4), ctypes.POINTER(Array4), ctypes.POINTER(Array4),
            ctypes.POINTER(Array4), ctypes.POINTER(Array4), ctypes.c_void_p, ctypes.POINTER(Array4),
            Box, ctypes.POINTER(ctypes.c_double), ctypes.c_uint, ctypes.c_void_p]
declare("ocfd_rhs_eb_box_f64_static_scratch", ctypes.c_int, argtypes)
L = ocfd.load()
ctx = ocfd.Context()
nx, ny, nz = 20, 18, 6
lo = (8, -4, 2); hi = (lo[0] + nx - 1, lo[1] + ny - 1, lo[2] + nz - 1); g4 = tuple(x - 4 for x in lo)
S = torch.from_numpy(inputs.ideal_state(nx, ny, nz, 41)).cuda()
geom = inputs.cylinder_box(nx, ny, nz)
dev = dict((k, torch.from_numpy(np.ascontiguousarray(geom[k])).cuda()) for k in ("vfrac", "apx", "apy", "apz"))
dev["flag"] = torch.from_numpy(np.ascontiguousarray(geom["flag"]).view(np.int32)).cuda()
dS = torch.zeros((5, nz, ny, nx), dtype=torch.float64, device="cuda")
aS, aD = ocfd.array4(S, g4), ocfd.array4(dS, lo)
af, av = ocfd.flag4(dev["flag"], g4), ocfd.array4(dev["vfrac"], g4)
ap = [ocfd.array4(dev[k], lo) for k in ("apx", "apy", "apz")]
dx = (ctypes.c_double * 3)(4.0, 4.0, 4.0)
stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
torch.cuda.synchronize()
free0, _ = torch.cuda.mem_get_info()
st = L.ocfd_rhs_eb_box_f64_static_scratch(ctx.h, ctypes.byref(aS), ctypes.byref(aD), None, ctypes.byref(af),
                                         ctypes.byref(av), ctypes.byref(ap[0]), ctypes.byref(ap[1]),
                                         ctypes.byref(ap[2]), None, None, ocfd.box(lo, hi), dx, 1, stream)
ocfd.check(st, "ocfd_rhs_eb_box_f64_static_scratch")
torch.cuda.synchronize()
free1, _ = torch.cuda.mem_get_info()
assert torch.isfinite(dS).all() and dS.abs().max() > 0
print("FREE", free0, free1)
"""


def test_first_call_in_fresh_process_allocates_nothing():
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    paths = ", ".join(repr(os.path.join(root, p)) for p in ("opencfd-amr_gb300", "tests", "oracle"))
    r = subprocess.run([sys.executable, "-c", _FRESH.format(paths=paths)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("FREE")][-1]
    free0, free1 = (int(x) for x in line.split()[1:])
    assert free1 == free0, (free0, free1)
