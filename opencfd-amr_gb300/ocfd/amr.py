"""AMR hierarchy binding (ocfd_amr_* in include/ocfd/ocfd.h): levels of ratio
2 advanced with subcycling, coarse-fine interpolation, reflux, average-down and
density-gradient regridding on the device."""
from __future__ import annotations

import ctypes

import numpy as np

from ._abi import Box, check, declare, load
from .context import _stream_ptr
from .level import NG, TIME_INTEGRATION, EbDesc, Level

MAX_LEVELS = 6


class AmrDesc(ctypes.Structure):
    _fields_ = [("nbox0", ctypes.c_int32), ("boxes0", ctypes.POINTER(Box)), ("domain", Box),
                ("lo_bc", ctypes.c_int32 * 3), ("hi_bc", ctypes.c_int32 * 3),
                ("dx", ctypes.c_double * 3), ("prob_lo", ctypes.c_double * 3),
                ("bc_case", ctypes.c_int32), ("case_params", ctypes.c_double * 16),
                ("max_level", ctypes.c_int32), ("blocking_factor", ctypes.c_int32 * 3),
                ("max_grid_size", ctypes.c_int32 * 3), ("n_error_buf", ctypes.c_int32),
                ("regrid_int", ctypes.c_int32), ("refine_dengrad", ctypes.c_double)]


class AmrReactDesc(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_double), ("chem_substeps", ctypes.c_int32), ("flags", ctypes.c_uint32)]


_vp = ctypes.c_void_p
declare("ocfd_amr_create", ctypes.c_int, [_vp, ctypes.POINTER(AmrDesc), ctypes.POINTER(_vp)])
declare("ocfd_amr_create_reacting", ctypes.c_int, [_vp, ctypes.POINTER(AmrDesc), ctypes.POINTER(AmrReactDesc),
                                                   ctypes.POINTER(_vp)])
declare("ocfd_amr_destroy", ctypes.c_int, [_vp])
declare("ocfd_amr_nlevels", ctypes.c_int, [_vp])
declare("ocfd_amr_level", _vp, [_vp, ctypes.c_int])
declare("ocfd_amr_get_grids", ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(Box), ctypes.c_int])
declare("ocfd_amr_regrid", ctypes.c_int, [_vp, ctypes.c_int, _vp])
declare("ocfd_amr_set_grids", ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int32),
                                             ctypes.POINTER(Box), _vp])
declare("ocfd_amr_average_down", ctypes.c_int, [_vp, _vp])
declare("ocfd_amr_fill_ghosts", ctypes.c_int, [_vp, _vp])
declare("ocfd_amr_advance", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double, ctypes.c_uint, _vp])
declare("ocfd_amr_time", ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), _vp])
declare("ocfd_amr_set_time", ctypes.c_int, [_vp, ctypes.c_double, _vp])
declare("ocfd_amr_set_stop_time", ctypes.c_int, [_vp, ctypes.c_double, _vp])
declare("ocfd_amr_cell_steps", ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)])
declare("ocfd_amr_launches_per_step", ctypes.c_int, [_vp])
declare("ocfd_amr_kernels_launched", ctypes.c_int64, [_vp])
declare("ocfd_amr_state_elems", ctypes.c_size_t, [_vp, ctypes.c_int])
declare("ocfd_amr_copy_in", ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp])
declare("ocfd_amr_copy_out", ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp])
declare("ocfd_amr_set_eb", ctypes.c_int, [_vp, ctypes.POINTER(EbDesc)])
declare("ocfd_amr_set_time_integration", ctypes.c_int, [_vp, ctypes.c_int32])
declare("ocfd_amr_valid_elems", ctypes.c_int64, [_vp, ctypes.c_int])
declare("ocfd_amr_copy_valid_in", ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp])
declare("ocfd_amr_copy_valid_out", ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp])
declare("ocfd_amr_autotune", ctypes.c_int, [_vp, ctypes.c_uint, ctypes.c_int, _vp])
declare("ocfd_amr_tuned", ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)])


def _boxes_array(boxes):
    bx = (Box * max(1, len(boxes)))()
    for i, (lo, hi) in enumerate(boxes):
        bx[i].lo[:] = list(lo)
        bx[i].hi[:] = list(hi)
    return bx


class Hierarchy:
    """A refined hierarchy over the level-0 `boxes0` of the domain 0..n0-1.
    react = dict(dt=..., chem_substeps=4, visc=True): a reacting hierarchy
    (5 + 9 components, ocfd_amr_create_reacting)."""

    def __init__(self, ctx, boxes0, n0, lo_bc, hi_bc, dx, prob_lo=(0.0, 0.0, 0.0), bc_case=0,
                 case_params=(), max_level=2, blocking_factor=(32, 32, 32), max_grid_size=(128, 128, 128),
                 n_error_buf=1, regrid_int=2, refine_dengrad=0.05, react=None):
        self.ctx = ctx
        self.ncomp = 14 if react else 5
        self.lib = load()
        self.n0 = tuple(n0)
        self.dx0 = tuple(dx)
        d = AmrDesc()
        bx = _boxes_array(boxes0)
        d.nbox0 = len(boxes0)
        d.boxes0 = bx
        d.domain.lo[:] = [0, 0, 0]
        d.domain.hi[:] = [n - 1 for n in n0]
        d.lo_bc[:] = list(lo_bc)
        d.hi_bc[:] = list(hi_bc)
        d.dx[:] = list(dx)
        d.prob_lo[:] = list(prob_lo)
        d.bc_case = bc_case
        for i, v in enumerate(case_params):
            d.case_params[i] = v
        d.max_level = max_level
        d.blocking_factor[:] = list(blocking_factor)
        d.max_grid_size[:] = list(max_grid_size)
        d.n_error_buf = n_error_buf
        d.regrid_int = regrid_int
        d.refine_dengrad = refine_dengrad
        self.desc = d
        h = ctypes.c_void_p()
        if react:
            r = AmrReactDesc()
            r.dt = react["dt"]
            r.chem_substeps = react.get("chem_substeps", 4)
            r.flags = (1 if react.get("visc", True) else 0) | (4 if react.get("flux_fp32", False) else 0)
            self.rdesc = r
            check(self.lib.ocfd_amr_create_reacting(ctx.h, ctypes.byref(d), ctypes.byref(r), ctypes.byref(h)),
                  "ocfd_amr_create_reacting")
        else:
            check(self.lib.ocfd_amr_create(ctx.h, ctypes.byref(d), ctypes.byref(h)), "ocfd_amr_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.ocfd_amr_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- structure --------------------------------------------------------
    def nlevels(self):
        return int(self.lib.ocfd_amr_nlevels(self.h))

    def domain(self, lev):
        return (0, 0, 0), tuple((n << lev) - 1 for n in self.n0)

    def dx(self, lev):
        return tuple(x / (1 << lev) for x in self.dx0)

    def grids(self, lev):
        n = self.lib.ocfd_amr_get_grids(self.h, lev, None, 0)
        if n < 0:
            raise IndexError(lev)
        bx = (Box * max(1, n))()
        self.lib.ocfd_amr_get_grids(self.h, lev, bx, n)
        return [(tuple(bx[i].lo), tuple(bx[i].hi)) for i in range(n)]

    def all_grids(self):
        return [self.grids(l) for l in range(self.nlevels())]

    def level(self, lev):
        h = self.lib.ocfd_amr_level(self.h, lev)
        if not h:
            raise IndexError(lev)
        lo, hi = self.domain(lev)
        return Level.wrap(self.ctx, h, self.grids(lev), lo, hi, ncomp=self.ncomp)

    def set_eb(self, desc):
        """Cut every level with an embedded body (ocfd.level.eb_desc(...))."""
        check(self.lib.ocfd_amr_set_eb(self.h, ctypes.byref(desc)), "ocfd_amr_set_eb")

    def set_time_integration(self, scheme):
        """Time integration of every level: "Euler", "RK2", "RK3" or 1 / 2 / 3."""
        order = TIME_INTEGRATION.get(scheme, scheme)
        check(self.lib.ocfd_amr_set_time_integration(self.h, int(order)), "ocfd_amr_set_time_integration")

    def box_classes(self, lev):
        return self.level(lev).box_classes()

    def autotune(self, flags=0, reps=5, stream=None):
        """Autotune every level's batched stage kernel (kept for later regrids)."""
        check(self.lib.ocfd_amr_autotune(self.h, flags, reps, _stream_ptr(stream)), "ocfd_amr_autotune")

    def tuned(self, lev):
        t, s = ctypes.c_int32(), ctypes.c_int32()
        if self.lib.ocfd_amr_tuned(self.h, lev, ctypes.byref(t), ctypes.byref(s)) != 0:
            raise IndexError(lev)
        return t.value, s.value

    # ---- regridding ---------------------------------------------------------
    def regrid(self, lbase=0, stream=None):
        check(self.lib.ocfd_amr_regrid(self.h, lbase, _stream_ptr(stream)), "ocfd_amr_regrid")

    def set_grids(self, grids, stream=None):
        """grids: box lists of levels 1.. (level 0 is fixed)."""
        nlev = 1 + len(grids)
        nbox = (ctypes.c_int32 * nlev)(*([0] + [len(g) for g in grids]))
        flat = [b for g in grids for b in g]
        bx = _boxes_array(flat)
        check(self.lib.ocfd_amr_set_grids(self.h, nlev, nbox, bx, _stream_ptr(stream)), "ocfd_amr_set_grids")

    def build(self, fab_of_box, stream=None):
        """Hierarchy at t = 0 (AMReX bldFineLevels): level 0 from the initial
        condition, then per level: tag, make the next level, set its initial
        condition; finally average down.  fab_of_box(lev, lo, hi, dx) returns the
        grown FAB of a box."""
        L0 = self.level(0)
        L0.copy_in(L0.pack_fabs(lambda lo, hi: fab_of_box(0, lo, hi, self.dx(0))), stream)
        for lev in range(self.desc.max_level):
            if self.nlevels() != lev + 1:
                break
            self.regrid(lev, stream)
            if self.nlevels() == lev + 2:
                L = self.level(lev + 1)
                L.copy_in(L.pack_fabs(lambda lo, hi, l=lev + 1: fab_of_box(l, lo, hi, self.dx(l))), stream)
        self.average_down(stream)
        self.set_time(0.0, stream)

    # ---- stepping -------------------------------------------------------------
    def average_down(self, stream=None):
        check(self.lib.ocfd_amr_average_down(self.h, _stream_ptr(stream)), "average_down")

    def fill_ghosts(self, stream=None):
        check(self.lib.ocfd_amr_fill_ghosts(self.h, _stream_ptr(stream)), "fill_ghosts")

    def advance(self, nsteps, cfl, flags=0, stream=None):
        check(self.lib.ocfd_amr_advance(self.h, nsteps, cfl, flags, _stream_ptr(stream)), "ocfd_amr_advance")

    def time(self, stream=None):
        t = ctypes.c_double()
        dt = ctypes.c_double()
        check(self.lib.ocfd_amr_time(self.h, ctypes.byref(t), ctypes.byref(dt), _stream_ptr(stream)), "time")
        return t.value, dt.value

    def set_time(self, t, stream=None):
        check(self.lib.ocfd_amr_set_time(self.h, t, _stream_ptr(stream)), "set_time")

    def set_stop_time(self, t, stream=None):
        check(self.lib.ocfd_amr_set_stop_time(self.h, t, _stream_ptr(stream)), "set_stop_time")

    def cell_steps(self):
        a = ctypes.c_int64()
        b = ctypes.c_int64()
        check(self.lib.ocfd_amr_cell_steps(self.h, ctypes.byref(a), ctypes.byref(b)), "cell_steps")
        return a.value, b.value

    def launches_per_step(self):
        return int(self.lib.ocfd_amr_launches_per_step(self.h))

    def kernels_launched(self):
        return int(self.lib.ocfd_amr_kernels_launched(self.h))

    # ---- data -----------------------------------------------------------------
    def level_global(self, lev, stream=None):
        """(valid data (5, Nz, Ny, Nx) of the whole level domain, mask of valid cells)"""
        L = self.level(lev)
        lo, hi = self.domain(lev)
        n = [hi[d] + 1 for d in range(3)]
        out = np.full((self.ncomp, n[2], n[1], n[0]), np.nan)
        L.unpack_valid(L.copy_out(stream=stream), out)
        mask = np.zeros((n[2], n[1], n[0]), bool)
        for blo, bhi in L.boxes:
            mask[blo[2]:bhi[2] + 1, blo[1]:bhi[1] + 1, blo[0]:bhi[0] + 1] = True
        return out, mask

    def state_elems(self, lev):
        return int(self.lib.ocfd_amr_state_elems(self.h, lev))

    def copy_in(self, lev, buf, stream=None):
        """buf: host numpy array or CUDA tensor of state_elems(lev) doubles."""
        ptr = buf.ctypes.data if isinstance(buf, np.ndarray) else buf.data_ptr()
        check(self.lib.ocfd_amr_copy_in(self.h, lev, ctypes.c_void_p(ptr), _stream_ptr(stream)), "amr copy_in")

    def copy_out(self, lev, buf=None, stream=None):
        if buf is None:
            buf = np.empty(self.state_elems(lev))
        ptr = buf.ctypes.data if isinstance(buf, np.ndarray) else buf.data_ptr()
        check(self.lib.ocfd_amr_copy_out(self.h, lev, ctypes.c_void_p(ptr), _stream_ptr(stream)), "amr copy_out")
        return buf

    def valid_elems(self, lev):
        return int(self.lib.ocfd_amr_valid_elems(self.h, lev))

    def copy_valid_in(self, lev, buf, stream=None):
        """buf: host numpy array or CUDA tensor of valid_elems(lev) doubles (the
        level's valid cells box after box, (5, nz, ny, nx) each)."""
        ptr = buf.ctypes.data if isinstance(buf, np.ndarray) else buf.data_ptr()
        check(self.lib.ocfd_amr_copy_valid_in(self.h, lev, ctypes.c_void_p(ptr), _stream_ptr(stream)),
              "amr copy_valid_in")

    def copy_valid_out(self, lev, buf=None, stream=None):
        if buf is None:
            buf = np.empty(self.valid_elems(lev))
        ptr = buf.ctypes.data if isinstance(buf, np.ndarray) else buf.data_ptr()
        check(self.lib.ocfd_amr_copy_valid_out(self.h, lev, ctypes.c_void_p(ptr), _stream_ptr(stream)),
              "amr copy_valid_out")
        return buf

    def snapshot(self):
        """Grids, state and time of every level (host), for restore()."""
        import torch
        data = [self.copy_out(l) for l in range(self.nlevels())]
        torch.cuda.synchronize()
        return dict(grids=self.all_grids(), data=data, time=self.time()[0])

    def restore(self, snap, stream=None):
        import torch
        self.set_grids(snap["grids"][1:], stream)
        for l, d in enumerate(snap["data"]):
            self.copy_in(l, d, stream)
        torch.cuda.synchronize()
        self.set_time(snap["time"], stream)
