"""ctypes bindings for the CPU oracle (test infrastructure).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module, and only to check or time against it.  Two libraries are bound:

* ``Oracle``    - the plain-C restatement (oracle/ocfd_oracle.c), built on any
  machine by ``make -C oracle``;
* ``RefOracle`` - OpenCFD-AMR's own kernel headers compiled from the reference
  sources (``make -C oracle ref``); present only where the reference tree is.

Arrays follow the oracle convention (see ocfd_oracle.h): numpy arrays shaped
(ncomp, z, y, x), C-contiguous float64, cell arrays over the box grown by NG.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
NG = 4
NSPEC = 9
_dp = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "oracle arrays must be C-contiguous"
    return a.ctypes.data_as(ctypes.c_void_p)


class ParmStruct(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in (
        "eos_gamma", "eos_m", "Patm", "cv", "cp", "Ru", "Rg", "kOverMu",
        "Pr", "C_s", "T_s", "smallr", "smallp", "eps", "twoThirds", "oneSix")] + [
        ("mw", ctypes.c_double * NSPEC),
        ("nasa_lo", (ctypes.c_double * 7) * NSPEC),
        ("nasa_hi", (ctypes.c_double * 7) * NSPEC),
        ("HP", ctypes.c_double * NSPEC),
        ("A0", ctypes.c_double * NSPEC),
        ("visccoeff", ctypes.c_double * (NSPEC * 5)),
        ("conductcoeff", ctypes.c_double * (NSPEC * 5)),
        ("diffcoeff", ctypes.c_double * (45 * 5)),
    ]


class BCStruct(ctypes.Structure):
    _fields_ = [("lo_bc", ctypes.c_int * 3), ("hi_bc", ctypes.c_int * 3),
                ("dirichlet_case", ctypes.c_int),
                ("prob_lo", ctypes.c_double * 3), ("dx", ctypes.c_double * 3),
                ("dom_lo", ctypes.c_int * 3), ("dom_hi", ctypes.c_int * 3),
                ("dmr_left", ctypes.c_double * 5), ("dmr_right", ctypes.c_double * 5),
                ("jet", ctypes.c_double * 8)]


def build_oracle(quiet=True):
    """Compile the restatement (and, where the reference tree exists, the
    reference build).  Returns the path of liboracle.so."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return os.path.join(HERE, "_build", "liboracle.so")


def reference_dir():
    """Root of the OpenCFD-AMR source tree the reference build compiles from:
    $OCFD_REFERENCE_DIR, else the tree this build was pinned against (the
    ``REF`` default of oracle/Makefile); None where neither holds the sources
    (machines without the reference, e.g. the GPU host)."""
    d = os.environ.get("OCFD_REFERENCE_DIR") or _MAKEFILE_REF
    return d if os.path.isdir(os.path.join(d, "Source")) else None


def _makefile_ref():
    with open(os.path.join(HERE, "Makefile")) as f:
        for line in f:
            if line.startswith("REF") and "?=" in line:
                return line.split("?=", 1)[1].strip()
    return ""


_MAKEFILE_REF = _makefile_ref()


def build_ref():
    """Build oracle/_ref from the reference sources, if they are present."""
    ref = reference_dir()
    if ref is None:
        return False
    out = subprocess.run(["make", "-C", HERE, "ref", "REF=" + ref], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference build failed:\n" + out.stdout + out.stderr)
    return True


def grown_shape(nc, nx, ny, nz):
    return (nc, nz + 2 * NG, ny + 2 * NG, nx + 2 * NG)


def face_shape(nc, nx, ny, nz, d):
    return (nc, nz + (d == 2), ny + (d == 1), nx + (d == 0))


class Oracle:
    """The plain-C restatement."""

    def __init__(self, path=None, openmp=False, fast=False):
        """openmp: the OpenMP build (same results); fast: the -O3 serial build
        with FMA contraction, for timing only (its results are not the oracle's)."""
        if path is None:
            build_oracle()
            name = "liboracle_fast.so" if fast else ("liboracle_omp.so" if openmp else "liboracle.so")
            path = os.path.join(HERE, "_build", name)
        self.lib = ctypes.CDLL(path)
        L = self.lib
        L.ocfdo_estdt.restype = ctypes.c_double
        L.ocfdo_advance_rk3.restype = ctypes.c_double
        L.ocfdo_advance_rk12.restype = ctypes.c_double
        for n in ("ckrhoy", "ckubms", "ckcvbs", "ckpy", "get_t_given_ey"):
            getattr(L, "ocfdo_" + n).restype = ctypes.c_double
        L.ocfdo_ckrhoy.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_void_p]
        L.ocfdo_ckubms.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p]
        L.ocfdo_ckcvbs.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p]
        L.ocfdo_ckpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double]
        L.ocfdo_get_t_given_ey.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p]
        L.ocfdo_production_rate.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                                            ctypes.c_void_p, ctypes.c_void_p]
        L.ocfdo_mixture_properties.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_void_p]
        L.ocfdo_mix_diff_coeffs.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_void_p, ctypes.c_void_p]
        L.ocfdo_species_enthalpy.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p]
        L.ocfdo_chem_advance.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_longlong, ctypes.c_longlong, ctypes.c_double]
        L.ocfdo_spec_renorm.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong,
                                        ctypes.c_longlong]
        L.ocfdo_fill_ghosts.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.ocfdo_advance_rk3.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.ocfdo_advance_rk12.argtypes = L.ocfdo_advance_rk3.argtypes
        self.parm = ParmStruct()
        L.ocfdo_parm_default(ctypes.byref(self.parm))
        self.pp = ctypes.cast(ctypes.byref(self.parm), ctypes.c_void_p)

    # -- box level ---------------------------------------------------------
    def c2prim(self, S, spec=None):
        nc, gz, gy, gx = S.shape
        nx, ny, nz = gx - 2 * NG, gy - 2 * NG, gz - 2 * NG
        chem = spec is not None
        q = np.zeros((8 if chem else 7, gz, gy, gx))
        self.lib.ocfdo_c2prim(self.pp, int(chem), _ptr(S), _ptr(spec), nx, ny, nz, _ptr(q))
        return q

    def rhs_regular(self, S, dxinv, do_visc=False, do_gravity=False):
        _, gz, gy, gx = S.shape
        nx, ny, nz = gx - 2 * NG, gy - 2 * NG, gz - 2 * NG
        dS = np.zeros((5, nz, ny, nx))
        f = [np.zeros(face_shape(5, nx, ny, nz, d)) for d in range(3)]
        dx = (ctypes.c_double * 3)(*dxinv)
        self.lib.ocfdo_rhs_regular(self.pp, _ptr(S), nx, ny, nz, dx, int(bool(do_visc)) | (2 if do_gravity else 0),
                                   _ptr(dS),
                                   _ptr(f[0]), _ptr(f[1]), _ptr(f[2]))
        return dS, f

    def rhs_eb(self, S, geom, dxinv, do_visc=False, do_redistribute=False):
        _, gz, gy, gx = S.shape
        nx, ny, nz = gx - 2 * NG, gy - 2 * NG, gz - 2 * NG
        dS = np.zeros((5, nz, ny, nx))
        f = [np.zeros(face_shape(5, nx, ny, nz, d)) for d in range(3)]
        dx = (ctypes.c_double * 3)(*dxinv)
        self.lib.ocfdo_rhs_eb(self.pp, _ptr(S), _ptr(geom["flag"]), _ptr(geom["vfrac"]),
                              _ptr(geom["apx"]), _ptr(geom["apy"]), _ptr(geom["apz"]),
                              nx, ny, nz, dx, int(do_visc), int(do_redistribute), _ptr(dS),
                              _ptr(f[0]), _ptr(f[1]), _ptr(f[2]))
        return dS, f

    def rhs_chem(self, S, spec, dxinv, do_visc=True, geom=None):
        _, gz, gy, gx = S.shape
        nx, ny, nz = gx - 2 * NG, gy - 2 * NG, gz - 2 * NG
        dS = np.zeros((5, nz, ny, nx))
        dSs = np.zeros((NSPEC, nz, ny, nx))
        f = [np.zeros(face_shape(5, nx, ny, nz, d)) for d in range(3)]
        fs = [np.zeros(face_shape(NSPEC, nx, ny, nz, d)) for d in range(3)]
        fd = [np.zeros(face_shape(NSPEC, nx, ny, nz, d)) for d in range(3)]
        dx = (ctypes.c_double * 3)(*dxinv)
        if geom is None:
            self.lib.ocfdo_rhs_chem(self.pp, _ptr(S), _ptr(spec), nx, ny, nz, dx, int(do_visc),
                                    _ptr(dS), _ptr(dSs), *[_ptr(a) for a in f + fs + fd])
        else:
            self.lib.ocfdo_rhs_chem_eb(self.pp, _ptr(S), _ptr(spec), _ptr(geom["flag"]),
                                       _ptr(geom["vfrac"]), _ptr(geom["apx"]), _ptr(geom["apy"]),
                                       _ptr(geom["apz"]), nx, ny, nz, dx, int(do_visc), _ptr(dS),
                                       _ptr(dSs), *[_ptr(a) for a in f + fs + fd])
        return dS, dSs, f, fs, fd

    def transport(self, S, spec):
        _, gz, gy, gx = S.shape
        nx, ny, nz = gx - 2 * NG, gy - 2 * NG, gz - 2 * NG
        mu = np.zeros((1, gz, gy, gx)); lam = np.zeros_like(mu)
        D = np.zeros((NSPEC, gz, gy, gx))
        self.lib.ocfdo_transport(self.pp, _ptr(S), _ptr(spec), nx, ny, nz, _ptr(mu), _ptr(lam), _ptr(D))
        return mu, lam, D

    def estdt(self, S, dx):
        _, gz, gy, gx = S.shape
        d = (ctypes.c_double * 3)(*dx)
        return self.lib.ocfdo_estdt(self.pp, _ptr(S), gx - 2 * NG, gy - 2 * NG, gz - 2 * NG, d)

    def chem_advance(self, S, spec, dt):
        """In place on (5, ncell) / (9, ncell) arrays."""
        assert S.shape[1] == spec.shape[1]
        self.lib.ocfdo_chem_advance(self.pp, _ptr(S), _ptr(spec), S.shape[1], S.shape[1], dt)

    def spec_renorm(self, S, spec):
        self.lib.ocfdo_spec_renorm(_ptr(S), _ptr(spec), S.shape[1], S.shape[1])

    # -- thermochemistry points ------------------------------------------------
    def ckxty(self, x):
        x = np.ascontiguousarray(x, float); y = np.zeros(NSPEC)
        self.lib.ocfdo_ckxty(self.pp, _ptr(x), _ptr(y)); return y

    def ckytx(self, y):
        y = np.ascontiguousarray(y, float); x = np.zeros(NSPEC)
        self.lib.ocfdo_ckytx(self.pp, _ptr(y), _ptr(x)); return x

    def ckrhoy(self, P, T, y):
        return self.lib.ocfdo_ckrhoy(self.pp, P, T, _ptr(np.ascontiguousarray(y, float)))

    def ckubms(self, T, rhoi):
        return self.lib.ocfdo_ckubms(self.pp, T, _ptr(np.ascontiguousarray(rhoi, float)))

    def ckpy(self, rhoi, T):
        return self.lib.ocfdo_ckpy(self.pp, _ptr(np.ascontiguousarray(rhoi, float)), T)

    def get_t_given_ey(self, e, rhoi):
        return self.lib.ocfdo_get_t_given_ey(self.pp, e, _ptr(np.ascontiguousarray(rhoi, float)))

    def production_rate(self, c, T):
        c = np.ascontiguousarray(c, float); w = np.zeros(NSPEC); A = np.zeros((NSPEC, NSPEC))
        self.lib.ocfdo_production_rate(self.pp, _ptr(c), T, _ptr(w), _ptr(A)); return w, A

    def gauss(self, A, b):
        A = np.ascontiguousarray(A, float); b = np.ascontiguousarray(b, float); x = np.zeros(NSPEC)
        self.lib.ocfdo_gauss(_ptr(A), _ptr(b), _ptr(x)); return x

    def mixture_properties(self, T, X):
        mu = ctypes.c_double(); lam = ctypes.c_double()
        self.lib.ocfdo_mixture_properties(self.pp, T, _ptr(np.ascontiguousarray(X, float)),
                                          ctypes.byref(mu), ctypes.byref(lam))
        return mu.value, lam.value

    def mix_diff_coeffs(self, T, P, X):
        D = np.zeros(NSPEC)
        self.lib.ocfdo_mix_diff_coeffs(self.pp, T, P, _ptr(np.ascontiguousarray(X, float)), _ptr(D))
        return D

    def species_enthalpy(self, T):
        h = np.zeros(NSPEC); self.lib.ocfdo_species_enthalpy(self.pp, T, _ptr(h)); return h

    # -- single-box time stepping ------------------------------------------------
    def fill_ghosts(self, bc, S, time=0.0):
        nc, gz, gy, gx = S.shape
        self.lib.ocfdo_fill_ghosts(ctypes.byref(bc), _ptr(S), nc, gx - 2 * NG, gy - 2 * NG,
                                   gz - 2 * NG, time)

    def advance_rk3(self, bc, S, cfl, nsteps, form=0, do_visc=False, do_gravity=False):
        _, gz, gy, gx = S.shape
        dts = np.zeros(nsteps)
        t = self.lib.ocfdo_advance_rk3(self.pp, ctypes.byref(bc), _ptr(S), gx - 2 * NG,
                                       gy - 2 * NG, gz - 2 * NG, int(bool(do_visc)) | (2 if do_gravity else 0),
                                       cfl, nsteps, form,
                                       _ptr(dts))
        return t, dts

    def box_rk3_step(self, S, dxinv, dt, geom=None, do_redistribute=False):
        """One SSP-RK3 step of one grown box in place, no ghost exchange between
        stages (the timed unit of the CPU baseline); geom: cut-cell data as for
        rhs_eb, None for the regular scheme."""
        _, gz, gy, gx = S.shape
        dx = (ctypes.c_double * 3)(*dxinv)
        g = geom or {}
        self.lib.ocfdo_box_rk3_step(self.pp, _ptr(S), _ptr(g.get("flag")), _ptr(g.get("vfrac")),
                                    _ptr(g.get("apx")), _ptr(g.get("apy")), _ptr(g.get("apz")),
                                    gx - 2 * NG, gy - 2 * NG, gz - 2 * NG, dx, int(do_redistribute),
                                    ctypes.c_double(dt))

    def advance_rk(self, bc, S, cfl, nsteps, order, do_visc=False):
        """nsteps of ebr.time_integration = "Euler" (order 1), "RK2" (2) or RK3 (3,
        Shu-Osher form) on a ghost-grown state, in place."""
        if order == 3:
            return self.advance_rk3(bc, S, cfl, nsteps, form=1, do_visc=do_visc)
        _, gz, gy, gx = S.shape
        dts = np.zeros(nsteps)
        t = self.lib.ocfdo_advance_rk12(self.pp, ctypes.byref(bc), _ptr(S), gx - 2 * NG,
                                        gy - 2 * NG, gz - 2 * NG, int(do_visc), cfl, nsteps, order,
                                        _ptr(dts))
        return t, dts


class RefOracle:
    """OpenCFD-AMR's own kernels, compiled from the reference sources."""

    def __init__(self):
        self.ideal = ctypes.CDLL(os.path.join(HERE, "_ref", "libocfd_ref_ideal.so"))
        self.chem = ctypes.CDLL(os.path.join(HERE, "_ref", "libocfd_ref_chem.so"))
        for L in (self.ideal, self.chem):
            L.ocfdr_estdt.restype = ctypes.c_double
        C = self.chem
        for n in ("ckrhoy", "ckubms", "ckpy", "get_t_given_ey"):
            getattr(C, "ocfdr_" + n).restype = ctypes.c_double
        C.ocfdr_ckrhoy.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_void_p]
        C.ocfdr_ckubms.argtypes = [ctypes.c_double, ctypes.c_void_p]
        C.ocfdr_ckpy.argtypes = [ctypes.c_void_p, ctypes.c_double]
        C.ocfdr_get_t_given_ey.argtypes = [ctypes.c_double, ctypes.c_void_p]
        C.ocfdr_production_rate.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p,
                                            ctypes.c_void_p]
        C.ocfdr_mixture_properties.argtypes = [ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_void_p]
        C.ocfdr_mix_diff_coeffs.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
                                            ctypes.c_void_p]
        C.ocfdr_species_enthalpy.argtypes = [ctypes.c_double, ctypes.c_void_p]
        C.ocfdr_chem_advance.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong,
                                         ctypes.c_longlong, ctypes.c_double]

    @staticmethod
    def available():
        return all(os.path.exists(os.path.join(HERE, "_ref", f))
                   for f in ("libocfd_ref_ideal.so", "libocfd_ref_chem.so"))

    def parm_scalars(self, chem=False):
        d = (ctypes.c_double * 16)()
        (self.chem if chem else self.ideal).ocfdr_parm_scalars(d)
        return list(d)

    def chem_tables(self):
        mw = np.zeros(9); lo = np.zeros(63); hi = np.zeros(63); hp = np.zeros(9); a0 = np.zeros(9)
        visc = np.zeros(45); cond = np.zeros(45); diff = np.zeros(225)
        self.chem.ocfdr_chem_tables(*[_ptr(a) for a in (mw, lo, hi, hp, a0, visc, cond, diff)])
        return dict(mw=mw, lo=lo.reshape(9, 7), hi=hi.reshape(9, 7), HP=hp, A0=a0, visc=visc,
                    cond=cond, diff=diff)

    def c2prim(self, S, spec=None):
        nc, gz, gy, gx = S.shape
        L = self.chem if spec is not None else self.ideal
        q = np.zeros((8 if spec is not None else 7, gz, gy, gx))
        L.ocfdr_c2prim(_ptr(S), _ptr(spec), gx - 2 * NG, gy - 2 * NG, gz - 2 * NG, _ptr(q))
        return q

    def rhs_regular(self, S, dxinv, do_visc=False):
        _, gz, gy, gx = S.shape
        nx, ny, nz = gx - 2 * NG, gy - 2 * NG, gz - 2 * NG
        dS = np.zeros((5, nz, ny, nx))
        f = [np.zeros(face_shape(5, nx, ny, nz, d)) for d in range(3)]
        dx = (ctypes.c_double * 3)(*dxinv)
        self.ideal.ocfdr_rhs_regular(_ptr(S), nx, ny, nz, dx, int(do_visc), _ptr(dS),
                                     _ptr(f[0]), _ptr(f[1]), _ptr(f[2]))
        return dS, f

    def rhs_eb(self, S, geom, dxinv, do_visc=False, do_redistribute=False):
        _, gz, gy, gx = S.shape
        nx, ny, nz = gx - 2 * NG, gy - 2 * NG, gz - 2 * NG
        dS = np.zeros((5, nz, ny, nx))
        f = [np.zeros(face_shape(5, nx, ny, nz, d)) for d in range(3)]
        dx = (ctypes.c_double * 3)(*dxinv)
        self.ideal.ocfdr_rhs_eb(_ptr(S), _ptr(geom["flag"]), _ptr(geom["vfrac"]),
                                _ptr(geom["apx"]), _ptr(geom["apy"]), _ptr(geom["apz"]),
                                nx, ny, nz, dx, int(do_visc), int(do_redistribute), _ptr(dS),
                                _ptr(f[0]), _ptr(f[1]), _ptr(f[2]))
        return dS, f

    def rhs_chem(self, S, spec, dxinv, do_visc=True, geom=None):
        _, gz, gy, gx = S.shape
        nx, ny, nz = gx - 2 * NG, gy - 2 * NG, gz - 2 * NG
        dS = np.zeros((5, nz, ny, nx))
        dSs = np.zeros((NSPEC, nz, ny, nx))
        f = [np.zeros(face_shape(5, nx, ny, nz, d)) for d in range(3)]
        fs = [np.zeros(face_shape(NSPEC, nx, ny, nz, d)) for d in range(3)]
        fd = [np.zeros(face_shape(NSPEC, nx, ny, nz, d)) for d in range(3)]
        dx = (ctypes.c_double * 3)(*dxinv)
        if geom is None:
            self.chem.ocfdr_rhs_chem(_ptr(S), _ptr(spec), nx, ny, nz, dx, int(do_visc), _ptr(dS),
                                     _ptr(dSs), *[_ptr(a) for a in f + fs + fd])
        else:
            self.chem.ocfdr_rhs_chem_eb(_ptr(S), _ptr(spec), _ptr(geom["flag"]),
                                        _ptr(geom["vfrac"]), _ptr(geom["apx"]),
                                        _ptr(geom["apy"]), _ptr(geom["apz"]), nx, ny, nz, dx,
                                        int(do_visc), _ptr(dS), _ptr(dSs),
                                        *[_ptr(a) for a in f + fs + fd])
        return dS, dSs, f, fs, fd

    def transport(self, S, spec):
        _, gz, gy, gx = S.shape
        mu = np.zeros((1, gz, gy, gx)); lam = np.zeros_like(mu); D = np.zeros((NSPEC, gz, gy, gx))
        self.chem.ocfdr_transport(_ptr(S), _ptr(spec), gx - 2 * NG, gy - 2 * NG, gz - 2 * NG,
                                  _ptr(mu), _ptr(lam), _ptr(D))
        return mu, lam, D

    def estdt(self, S, dx, chem=False):
        _, gz, gy, gx = S.shape
        d = (ctypes.c_double * 3)(*dx)
        return (self.chem if chem else self.ideal).ocfdr_estdt(_ptr(S), gx - 2 * NG, gy - 2 * NG,
                                                               gz - 2 * NG, d)

    def chem_advance(self, S, spec, dt):
        self.chem.ocfdr_chem_advance(_ptr(S), _ptr(spec), S.shape[1], S.shape[1], dt)

    def ckxty(self, x):
        x = np.ascontiguousarray(x, float); y = np.zeros(NSPEC)
        self.chem.ocfdr_ckxty(_ptr(x), _ptr(y)); return y

    def ckrhoy(self, P, T, y):
        return self.chem.ocfdr_ckrhoy(P, T, _ptr(np.ascontiguousarray(y, float)))

    def ckubms(self, T, rhoi):
        return self.chem.ocfdr_ckubms(T, _ptr(np.ascontiguousarray(rhoi, float)))

    def ckpy(self, rhoi, T):
        return self.chem.ocfdr_ckpy(_ptr(np.ascontiguousarray(rhoi, float)), T)

    def get_t_given_ey(self, e, rhoi):
        return self.chem.ocfdr_get_t_given_ey(e, _ptr(np.ascontiguousarray(rhoi, float)))

    def production_rate(self, c, T):
        c = np.ascontiguousarray(c, float); w = np.zeros(NSPEC); A = np.zeros((NSPEC, NSPEC))
        self.chem.ocfdr_production_rate(_ptr(c), T, _ptr(w), _ptr(A)); return w, A

    def gauss(self, A, b):
        A = np.ascontiguousarray(A, float); b = np.ascontiguousarray(b, float); x = np.zeros(NSPEC)
        self.chem.ocfdr_gauss(_ptr(A), _ptr(b), _ptr(x)); return x

    def mixture_properties(self, T, X):
        mu = ctypes.c_double(); lam = ctypes.c_double()
        self.chem.ocfdr_mixture_properties(T, _ptr(np.ascontiguousarray(X, float)),
                                           ctypes.byref(mu), ctypes.byref(lam))
        return mu.value, lam.value

    def mix_diff_coeffs(self, T, P, X):
        D = np.zeros(NSPEC)
        self.chem.ocfdr_mix_diff_coeffs(T, P, _ptr(np.ascontiguousarray(X, float)), _ptr(D))
        return D

    def species_enthalpy(self, T):
        h = np.zeros(NSPEC); self.chem.ocfdr_species_enthalpy(T, _ptr(h)); return h
