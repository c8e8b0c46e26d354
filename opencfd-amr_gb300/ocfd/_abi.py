"""ctypes declarations mirroring include/ocfd/ocfd.h."""
from __future__ import annotations

import ctypes
import os

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "_build", "libocfd.so")

c_double_p = ctypes.POINTER(ctypes.c_double)


class Array4(ctypes.Structure):
    """amrex::Array4<double> layout."""
    _fields_ = [("p", ctypes.c_void_p), ("jstride", ctypes.c_int64), ("kstride", ctypes.c_int64),
                ("nstride", ctypes.c_int64), ("begin", ctypes.c_int32 * 3),
                ("end", ctypes.c_int32 * 3), ("ncomp", ctypes.c_int32)]


class Flag4(Array4):
    """amrex::Array4<EBCellFlag const> layout (32-bit words)."""


class Box(ctypes.Structure):
    _fields_ = [("lo", ctypes.c_int32 * 3), ("hi", ctypes.c_int32 * 3)]


_PARM_SCALARS = ("eos_gamma", "eos_m", "Patm", "cv", "cp", "Ru", "Rg", "kOverMu", "Pr", "C_s",
                 "T_s", "smallr", "smallp", "eps", "twoThirds", "oneSix")
_PARM_TABLES = ("mw", "H2_lo", "H2_hi", "O2_lo", "O2_hi", "H2O_lo", "H2O_hi", "H_lo", "H_hi",
                "O_lo", "O_hi", "OH_lo", "OH_hi", "HO2_lo", "HO2_hi", "H2O2_lo", "H2O2_hi",
                "N2_lo", "N2_hi", "HP", "A0", "visccoeff", "conductcoeff", "diffcoeff")


class Parm(ctypes.Structure):
    """Layout of the reference's Parm (Source/Constants.H:7-64, CHEM build)."""
    _fields_ = [(n, ctypes.c_double) for n in _PARM_SCALARS] + [(n, c_double_p) for n in _PARM_TABLES]

    SCALARS = _PARM_SCALARS
    TABLES = _PARM_TABLES


class OcfdError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (%d): %s" % (status_string(status), status, msg))
        self.status = status


_lib = None

# name -> (restype, argtypes)
_SIGS = {
    "ocfd_parm_default": (ctypes.c_int, [ctypes.POINTER(Parm)]),
    "ocfd_context_create": (ctypes.c_int, [ctypes.POINTER(Parm), ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "ocfd_context_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "ocfd_context_check": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32)]),
    "ocfd_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "ocfd_last_error": (ctypes.c_char_p, []),
    "ocfd_version": (ctypes.c_int, []),
    "ocfd_built_arch": (ctypes.c_int, []),
    "ocfd_rhs_regular_box_f64": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Array4), ctypes.POINTER(Array4),
                                                ctypes.POINTER(Array4), Box, ctypes.POINTER(ctypes.c_double),
                                                ctypes.c_uint, ctypes.c_void_p]),
    "ocfd_rhs_eb_box_f64": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Array4), ctypes.POINTER(Array4),
                                           ctypes.POINTER(Array4), ctypes.POINTER(Flag4), ctypes.POINTER(Array4),
                                           ctypes.POINTER(Array4), ctypes.POINTER(Array4), ctypes.POINTER(Array4),
                                           ctypes.c_void_p, ctypes.POINTER(Array4), Box,
                                           ctypes.POINTER(ctypes.c_double), ctypes.c_uint, ctypes.c_void_p]),
    "ocfd_chem_advance_box_f64": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Array4), ctypes.POINTER(Array4),
                                                 Box, ctypes.c_double, ctypes.c_void_p]),
    "ocfd_spec_renorm_box_f64": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Array4), ctypes.POINTER(Array4),
                                                Box, ctypes.c_void_p]),
    "ocfd_rhs_chem_box_f64": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Array4), ctypes.POINTER(Array4),
                                             ctypes.POINTER(Array4), ctypes.POINTER(Array4), ctypes.POINTER(Array4),
                                             ctypes.POINTER(Array4), Box, ctypes.POINTER(ctypes.c_double),
                                             ctypes.c_uint, ctypes.c_void_p]),
    "ocfd_rhs_chem_eb_box_f64": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Array4), ctypes.POINTER(Array4),
                                                ctypes.POINTER(Array4), ctypes.POINTER(Array4), ctypes.POINTER(Array4),
                                                ctypes.POINTER(Array4), ctypes.POINTER(Flag4), ctypes.POINTER(Array4),
                                                ctypes.POINTER(Array4), ctypes.POINTER(Array4), ctypes.POINTER(Array4),
                                                ctypes.c_void_p, ctypes.POINTER(Array4), Box,
                                                ctypes.POINTER(ctypes.c_double), ctypes.c_uint, ctypes.c_void_p]),
    "ocfd_measure_fma_peaks": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "ocfd_measure_ffma2_peak": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double)]),
    "ocfd_check_rcp_f64": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                          ctypes.c_void_p]),
    "ocfd_set_tma_staging": (None, [ctypes.c_int32]),
}


def load(path=None, build_if_missing=True):
    """Load libocfd.so (building it first when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError("libocfd.so not built: " + path)
        from .build import build
        build()
    L = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        f = getattr(L, name, None)
        if f is None:
            continue
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def lib():
    return load()


def declare(name, restype, argtypes):
    """Register a signature (used by modules that bind further entry points)."""
    _SIGS[name] = (restype, argtypes)
    if _lib is not None:
        f = getattr(_lib, name)
        f.restype = restype
        f.argtypes = argtypes


def status_string(s):
    try:
        return load().ocfd_status_string(s).decode()
    except OSError:
        return "status"


def check(status, what=""):
    if status != 0:
        msg = load().ocfd_last_error().decode()
        raise OcfdError(status, (what + ": " if what else "") + msg)


def array4(t, begin=(0, 0, 0)):
    """Array4 view of a C-contiguous (ncomp, nz, ny, nx) float64 CUDA tensor whose
    first element is cell `begin` (absolute i, j, k)."""
    assert t.dim() == 4 and t.is_contiguous()
    nc, nz, ny, nx = t.shape
    a = Array4()
    a.p = t.data_ptr()
    a.jstride = nx
    a.kstride = nx * ny
    a.nstride = nx * ny * nz
    a.begin[:] = list(begin)
    a.end[:] = [begin[0] + nx, begin[1] + ny, begin[2] + nz]
    a.ncomp = nc
    return a


def flag4(t, begin=(0, 0, 0)):
    assert t.dim() == 4 and t.is_contiguous()
    _, nz, ny, nx = t.shape
    a = Flag4()
    a.p = t.data_ptr()
    a.jstride = nx
    a.kstride = nx * ny
    a.nstride = nx * ny * nz
    a.begin[:] = list(begin)
    a.end[:] = [begin[0] + nx, begin[1] + ny, begin[2] + nz]
    a.ncomp = 1
    return a


def box(lo, hi):
    b = Box()
    b.lo[:] = list(lo)
    b.hi[:] = list(hi)
    return b
