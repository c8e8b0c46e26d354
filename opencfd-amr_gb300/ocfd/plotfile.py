"""Plotfiles (AMReX HyperCLaw-V1.1 layout) and their comparison: bindings of
ocfd_plotfile_* / ocfd_amr_write_plotfile (include/ocfd/ocfd.h)."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from ._abi import Box, check, declare, load

_vp = ctypes.c_void_p


class PlotLevel(ctypes.Structure):
    _fields_ = [("nbox", ctypes.c_int32), ("boxes", ctypes.POINTER(Box)), ("fabs", ctypes.POINTER(_vp)),
                ("dx", ctypes.c_double * 3), ("step", ctypes.c_int32)]


declare("ocfd_plotfile_write", ctypes.c_int, [ctypes.c_char_p, ctypes.c_int32, ctypes.POINTER(PlotLevel),
                                              ctypes.c_int32, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(Box),
                                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                              ctypes.c_int32, ctypes.c_double])
declare("ocfd_plotfile_info", ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int32),
                                             ctypes.POINTER(ctypes.c_int32)])
declare("ocfd_plotfile_compare", ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int32, ctypes.c_int32,
                                                ctypes.c_int32, ctypes.POINTER(ctypes.c_double),
                                                ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32),
                                                ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)])
declare("ocfd_amr_write_plotfile", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_int32, _vp])


def write(path, levels, names, domain_hi, prob_lo, prob_hi, time=0.0, domain_lo=(0, 0, 0)):
    """levels: list of dict(boxes=[(lo, hi)], fabs=[array (ncomp, nz, ny, nx)], dx=(3), step=int)."""
    L = load()
    keep = []
    lv = (PlotLevel * len(levels))()
    for l, d in enumerate(levels):
        bx = (Box * len(d["boxes"]))()
        ptrs = (_vp * len(d["boxes"]))()
        for b, ((lo, hi), f) in enumerate(zip(d["boxes"], d["fabs"])):
            bx[b].lo[:] = list(lo)
            bx[b].hi[:] = list(hi)
            a = np.ascontiguousarray(f, dtype=np.float64)
            assert a.shape == (len(names), hi[2] - lo[2] + 1, hi[1] - lo[1] + 1, hi[0] - lo[0] + 1)
            keep.append(a)
            ptrs[b] = a.ctypes.data
        keep += [bx, ptrs]
        lv[l].nbox = len(d["boxes"])
        lv[l].boxes = bx
        lv[l].fabs = ptrs
        lv[l].dx[:] = list(d["dx"])
        lv[l].step = int(d.get("step", 0))
    nm = (ctypes.c_char_p * len(names))(*[n.encode() for n in names])
    dom = Box()
    dom.lo[:] = list(domain_lo)
    dom.hi[:] = list(domain_hi)
    check(L.ocfd_plotfile_write(os.fsencode(path), len(levels), lv, len(names), nm, ctypes.byref(dom),
                                (ctypes.c_double * 3)(*prob_lo), (ctypes.c_double * 3)(*prob_hi), 2, time),
          "ocfd_plotfile_write")


def varnames(path):
    with open(os.path.join(path, "Header")) as f:
        f.readline()
        n = int(f.readline())
        return [f.readline().strip() for _ in range(n)]


def info(path):
    nlev = ctypes.c_int32()
    ncomp = ctypes.c_int32()
    check(load().ocfd_plotfile_info(os.fsencode(path), ctypes.byref(nlev), ctypes.byref(ncomp)), "ocfd_plotfile_info")
    return nlev.value, ncomp.value


def compare(a, b, norm=0, allow_diff_grids=False):
    """fcompare of two plotfiles: dict(names, abs[l][n], rel[l][n], nan[l][n])."""
    nlev, ncomp = info(a)
    cap = nlev * ncomp
    ab = (ctypes.c_double * cap)()
    rel = (ctypes.c_double * cap)()
    nan = (ctypes.c_int32 * cap)()
    nl = ctypes.c_int32()
    nc = ctypes.c_int32()
    check(load().ocfd_plotfile_compare(os.fsencode(a), os.fsencode(b), norm, int(allow_diff_grids), cap, ab, rel, nan,
                                       ctypes.byref(nl), ctypes.byref(nc)), "ocfd_plotfile_compare")
    shape = (nl.value, nc.value)
    return dict(names=varnames(a), abs=np.array(ab[:]).reshape(shape), rel=np.array(rel[:]).reshape(shape),
                nan=np.array(nan[:]).reshape(shape))


def write_hierarchy(H, path, step=0, stream=None):
    from .context import _stream_ptr
    check(load().ocfd_amr_write_plotfile(H.h, os.fsencode(path), step, _stream_ptr(stream)),
          "ocfd_amr_write_plotfile")
