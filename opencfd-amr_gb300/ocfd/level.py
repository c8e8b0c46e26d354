"""Level driver binding: boxes of one AMR level advanced on the device
(see ocfd_level_* in include/ocfd/ocfd.h)."""
from __future__ import annotations

import ctypes

import numpy as np

from ._abi import Array4, Box, Flag4, check, declare, load
from .context import _stream_ptr

NG = 4


class LevelDesc(ctypes.Structure):
    _fields_ = [("nbox", ctypes.c_int32), ("boxes", ctypes.POINTER(Box)), ("domain", Box),
                ("lo_bc", ctypes.c_int32 * 3), ("hi_bc", ctypes.c_int32 * 3),
                ("dx", ctypes.c_double * 3), ("prob_lo", ctypes.c_double * 3),
                ("bc_case", ctypes.c_int32), ("case_params", ctypes.c_double * 16),
                ("tile", ctypes.c_int32)]


_vp = ctypes.c_void_p
declare("ocfd_level_create", ctypes.c_int, [_vp, ctypes.POINTER(LevelDesc), ctypes.POINTER(_vp)])
declare("ocfd_level_destroy", ctypes.c_int, [_vp])
declare("ocfd_level_state", ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(Array4)])
declare("ocfd_level_copy_in", ctypes.c_int, [_vp, _vp, _vp])
declare("ocfd_level_copy_out", ctypes.c_int, [_vp, _vp, _vp])
declare("ocfd_level_state_elems", ctypes.c_size_t, [_vp])
declare("ocfd_level_copy_valid_in", ctypes.c_int, [_vp, _vp, _vp])
declare("ocfd_level_copy_valid_out", ctypes.c_int, [_vp, _vp, _vp])
declare("ocfd_level_valid_elems", ctypes.c_int64, [_vp])
declare("ocfd_level_fill_ghosts", ctypes.c_int, [_vp, ctypes.c_double, _vp])
declare("ocfd_level_advance", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double, ctypes.c_uint, _vp])
declare("ocfd_level_time", ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_double), _vp])
declare("ocfd_level_set_time", ctypes.c_int, [_vp, ctypes.c_double, _vp])
declare("ocfd_level_cells", ctypes.c_int64, [_vp])
declare("ocfd_level_set_stop_time", ctypes.c_int, [_vp, ctypes.c_double, _vp])
declare("ocfd_level_launches_per_step", ctypes.c_int, [_vp, ctypes.c_uint])
declare("ocfd_level_profile_part", ctypes.c_int, [_vp, ctypes.c_uint, ctypes.c_int, ctypes.c_int,
                                                  ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64),
                                                  _vp])
declare("ocfd_level_profile_stage", ctypes.c_int, [_vp, ctypes.c_uint, ctypes.c_int,
                                                   ctypes.POINTER(ctypes.c_double), _vp])

CASE_NONE, CASE_DMR, CASE_INFLOW = 0, 1, 2
EB_NONE, EB_CYLINDER_Z = 0, 1
BOX_REGULAR, BOX_CUT, BOX_COVERED = 0, 1, 2


class EbDesc(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("nsub", ctypes.c_int32), ("center", ctypes.c_double * 2),
                ("radius", ctypes.c_double), ("redistribute", ctypes.c_int32)]


def eb_desc(kind=EB_CYLINDER_Z, center=(0.5, 0.5), radius=0.1, nsub=16, redistribute=False):
    d = EbDesc()
    d.kind = kind
    d.nsub = nsub
    d.center[:] = list(center)
    d.radius = radius
    d.redistribute = 1 if redistribute else 0
    return d


declare("ocfd_level_set_eb", ctypes.c_int, [_vp, ctypes.POINTER(EbDesc)])
declare("ocfd_level_set_schedule", ctypes.c_int, [_vp, ctypes.c_int32, ctypes.c_int32])
declare("ocfd_level_set_time_integration", ctypes.c_int, [_vp, ctypes.c_int32])

# ebr.time_integration (Source/EBR.cpp:36): order of the level's RK scheme
TIME_INTEGRATION = {"Euler": 1, "RK2": 2, "RK3": 3}
declare("ocfd_level_autotune", ctypes.c_int, [_vp, ctypes.c_uint, ctypes.c_int, ctypes.POINTER(ctypes.c_int32),
                                              ctypes.POINTER(ctypes.c_int32), _vp])
declare("ocfd_level_box_classes", ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int32)])
declare("ocfd_level_eb_geometry_copy", ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, _vp, _vp])
declare("ocfd_level_eb_geometry", ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(Flag4), ctypes.POINTER(Array4),
                                                 ctypes.POINTER(Array4)])


def chop_domain(n, max_grid):
    """Split the domain (0..n-1 per direction) into boxes of at most max_grid cells."""
    cuts = []
    for d in range(3):
        m = max_grid[d] if hasattr(max_grid, "__len__") else max_grid
        edges = list(range(0, n[d], m)) + [n[d]]
        cuts.append([(edges[i], edges[i + 1] - 1) for i in range(len(edges) - 1)])
    boxes = []
    for (zl, zh) in cuts[2]:
        for (yl, yh) in cuts[1]:
            for (xl, xh) in cuts[0]:
                boxes.append(((xl, yl, zl), (xh, yh, zh)))
    return boxes


class Level:
    def __init__(self, ctx, boxes, domain_hi, lo_bc, hi_bc, dx, prob_lo=(0.0, 0.0, 0.0),
                 bc_case=CASE_NONE, case_params=(), tile=-1, domain_lo=(0, 0, 0), ncomp=5):
        self.ctx = ctx
        self.lib = load()
        self.boxes = [(tuple(lo), tuple(hi)) for lo, hi in boxes]
        self.ncomp = ncomp
        bx = (Box * len(boxes))()
        for i, (lo, hi) in enumerate(self.boxes):
            bx[i].lo[:] = list(lo)
            bx[i].hi[:] = list(hi)
        d = LevelDesc()
        d.nbox = len(boxes)
        d.boxes = bx
        d.domain.lo[:] = list(domain_lo)
        d.domain.hi[:] = list(domain_hi)
        d.lo_bc[:] = list(lo_bc)
        d.hi_bc[:] = list(hi_bc)
        d.dx[:] = list(dx)
        d.prob_lo[:] = list(prob_lo)
        d.bc_case = bc_case
        for i, v in enumerate(case_params):
            d.case_params[i] = v
        d.tile = tile
        self._boxes_keepalive = bx
        h = ctypes.c_void_p()
        check(self.lib.ocfd_level_create(ctx.h, ctypes.byref(d), ctypes.byref(h)), "ocfd_level_create")
        self.h = h
        self.elems = self.lib.ocfd_level_state_elems(h)
        self.domain_lo = tuple(domain_lo)
        self.domain_hi = tuple(domain_hi)

    @classmethod
    def wrap(cls, ctx, handle, boxes, domain_lo, domain_hi, ncomp=5):
        """A view of a level owned elsewhere (an AMR hierarchy); never destroyed here."""
        self = cls.__new__(cls)
        self.ctx = ctx
        self.lib = load()
        self.boxes = [(tuple(lo), tuple(hi)) for lo, hi in boxes]
        self.ncomp = ncomp
        self.h = ctypes.c_void_p(handle)
        self.owned = False
        self.elems = self.lib.ocfd_level_state_elems(self.h)
        self.domain_lo = tuple(domain_lo)
        self.domain_hi = tuple(domain_hi)
        return self

    def close(self):
        if self.h and getattr(self, "owned", True):
            self.lib.ocfd_level_destroy(self.h)
        self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- data movement ------------------------------------------------------
    def pack(self, G):
        """Concatenate the grown FABs of every box cut from a global grown array
        G of shape (ncomp, Nz+8, Ny+8, Nx+8) that starts at domain_lo - 4."""
        parts = []
        for lo, hi in self.boxes:
            sl = tuple(slice(lo[d] - self.domain_lo[d], hi[d] - self.domain_lo[d] + 2 * NG + 1)
                       for d in (2, 1, 0))
            parts.append(np.ascontiguousarray(G[(slice(None),) + sl]).ravel())
        return np.concatenate(parts)

    def unpack_valid(self, flat, out):
        """Write every box's valid cells from the FAB concatenation into the
        global array `out` (ncomp, Nz, Ny, Nx) indexed from domain_lo."""
        off = 0
        for lo, hi in self.boxes:
            n = [hi[d] - lo[d] + 1 for d in range(3)]
            shape = (self.ncomp, n[2] + 2 * NG, n[1] + 2 * NG, n[0] + 2 * NG)
            size = int(np.prod(shape))
            fab = flat[off:off + size].reshape(shape)
            off += size
            sl = tuple(slice(lo[d] - self.domain_lo[d], hi[d] - self.domain_lo[d] + 1) for d in (2, 1, 0))
            out[(slice(None),) + sl] = fab[:, NG:-NG, NG:-NG, NG:-NG]
        return out

    def copy_in(self, flat, stream=None):
        """flat: numpy array (host) or CUDA tensor (device) of self.elems doubles."""
        if isinstance(flat, np.ndarray):
            assert flat.dtype == np.float64 and flat.size == self.elems and flat.flags["C_CONTIGUOUS"]
            ptr = flat.ctypes.data
        else:
            assert flat.numel() == self.elems
            ptr = flat.data_ptr()
        check(self.lib.ocfd_level_copy_in(self.h, ctypes.c_void_p(ptr), _stream_ptr(stream)), "copy_in")
        self._sync(stream)

    def copy_out(self, flat=None, stream=None):
        if flat is None:
            flat = np.empty(self.elems)
        ptr = flat.ctypes.data if isinstance(flat, np.ndarray) else flat.data_ptr()
        check(self.lib.ocfd_level_copy_out(self.h, ctypes.c_void_p(ptr), _stream_ptr(stream)), "copy_out")
        self._sync(stream)
        return flat

    def valid_elems(self):
        return int(self.lib.ocfd_level_valid_elems(self.h))

    def copy_valid_in(self, flat, stream=None):
        """flat: host numpy array or CUDA tensor of valid_elems() doubles, the
        valid cells box after box, (ncomp, nz, ny, nx) each."""
        n = self.valid_elems()
        if isinstance(flat, np.ndarray):
            assert flat.dtype == np.float64 and flat.size == n and flat.flags["C_CONTIGUOUS"]
            ptr = flat.ctypes.data
        else:
            assert flat.numel() == n
            ptr = flat.data_ptr()
        check(self.lib.ocfd_level_copy_valid_in(self.h, ctypes.c_void_p(ptr), _stream_ptr(stream)),
              "copy_valid_in")
        self._sync(stream)

    def copy_valid_out(self, flat=None, stream=None):
        if flat is None:
            flat = np.empty(self.valid_elems())
        ptr = flat.ctypes.data if isinstance(flat, np.ndarray) else flat.data_ptr()
        check(self.lib.ocfd_level_copy_valid_out(self.h, ctypes.c_void_p(ptr), _stream_ptr(stream)),
              "copy_valid_out")
        self._sync(stream)
        return flat

    def _sync(self, stream):
        import torch
        if stream is None:
            torch.cuda.current_stream().synchronize()
        elif not isinstance(stream, int):
            stream.synchronize()

    def set_global(self, G, stream=None):
        self.copy_in(self.pack(G), stream)

    def pack_fabs(self, fab_of_box):
        """Concatenate fab_of_box(lo, hi) over the boxes: each returns the grown
        FAB (ncomp, nz+8, ny+8, nx+8) of the valid box lo..hi."""
        return np.concatenate([np.ascontiguousarray(fab_of_box(lo, hi), dtype=np.float64).ravel()
                               for lo, hi in self.boxes])

    def get_global(self, stream=None):
        n = [self.domain_hi[d] - self.domain_lo[d] + 1 for d in range(3)]
        out = np.zeros((self.ncomp, n[2], n[1], n[0]))
        return self.unpack_valid(self.copy_out(stream=stream), out)

    # ---- stepping -------------------------------------------------------------
    def advance(self, nsteps, cfl, flags=0, stream=None):
        check(self.lib.ocfd_level_advance(self.h, nsteps, cfl, flags, _stream_ptr(stream)), "advance")

    def time(self, stream=None):
        t = ctypes.c_double(); dt = ctypes.c_double()
        check(self.lib.ocfd_level_time(self.h, ctypes.byref(t), ctypes.byref(dt), _stream_ptr(stream)), "time")
        return t.value, dt.value

    def set_time(self, t, stream=None):
        check(self.lib.ocfd_level_set_time(self.h, t, _stream_ptr(stream)), "set_time")

    def set_stop_time(self, t, stream=None):
        check(self.lib.ocfd_level_set_stop_time(self.h, t, _stream_ptr(stream)), "set_stop_time")

    def cells(self):
        return int(self.lib.ocfd_level_cells(self.h))

    def launches_per_step(self, flags=0):
        return int(self.lib.ocfd_level_launches_per_step(self.h, flags))

    def profile_regular(self, flags=0, reps=10, stream=None):
        """(ms per launch of the regular boxes' tile kernel of a stage, the cells
        of the regular boxes)"""
        ms = ctypes.c_double()
        cells = ctypes.c_int64()
        check(self.lib.ocfd_level_profile_part(self.h, flags, 1, reps, ctypes.byref(ms), ctypes.byref(cells),
                                               _stream_ptr(stream)), "profile_regular")
        return ms.value, cells.value

    def profile_stage(self, flags=0, reps=10, stream=None):
        ms = ctypes.c_double()
        check(self.lib.ocfd_level_profile_stage(self.h, flags, reps, ctypes.byref(ms), _stream_ptr(stream)),
              "profile_stage")
        return ms.value

    def set_schedule(self, tile, sched=0):
        """Tile shape (index, -1: keep) and schedule of the batched stage kernel."""
        check(self.lib.ocfd_level_set_schedule(self.h, tile, sched), "ocfd_level_set_schedule")

    def autotune(self, flags=0, reps=5, stream=None):
        """Pick the fastest tile shape x schedule of the batched stage kernel;
        returns (tile, sched)."""
        t, s = ctypes.c_int32(), ctypes.c_int32()
        check(self.lib.ocfd_level_autotune(self.h, flags, reps, ctypes.byref(t), ctypes.byref(s), _stream_ptr(stream)),
              "ocfd_level_autotune")
        return t.value, s.value

    def set_time_integration(self, scheme):
        """"Euler", "RK2" (Heun, the reference's default) or "RK3" (SSP-RK3, the
        default here), or the order 1 / 2 / 3."""
        order = TIME_INTEGRATION.get(scheme, scheme)
        check(self.lib.ocfd_level_set_time_integration(self.h, int(order)), "ocfd_level_set_time_integration")

    # ---- embedded body ---------------------------------------------------------
    def set_eb(self, desc):
        """Cut the level with an embedded body (EbDesc); classifies the boxes."""
        check(self.lib.ocfd_level_set_eb(self.h, ctypes.byref(desc)), "ocfd_level_set_eb")

    def box_classes(self):
        out = (ctypes.c_int32 * len(self.boxes))()
        check(self.lib.ocfd_level_box_classes(self.h, out), "ocfd_level_box_classes")
        return list(out)

    def eb_geometry(self, ibox):
        """(flag, vfrac, apx, apy) of a box with cut-cell data as 2D numpy arrays
        (y, x) over grow(bx, 5) (apx one column wider, apy one row taller), and
        the (x, y) cell index of their first element."""
        fl, vf = Flag4(), Array4()
        ap = (Array4 * 3)()
        check(self.lib.ocfd_level_eb_geometry(self.h, ibox, ctypes.byref(fl), ctypes.byref(vf), ap),
              "ocfd_level_eb_geometry")
        gx, gy = fl.end[0] - fl.begin[0], fl.end[1] - fl.begin[1]
        flag = np.empty((gy, gx), np.uint32)
        vfrac = np.empty((gy, gx))
        apx = np.empty((gy, gx + 1))
        apy = np.empty((gy + 1, gx))
        check(self.lib.ocfd_level_eb_geometry_copy(self.h, ibox, flag.ctypes.data_as(ctypes.c_void_p),
                                                   vfrac.ctypes.data_as(ctypes.c_void_p),
                                                   apx.ctypes.data_as(ctypes.c_void_p),
                                                   apy.ctypes.data_as(ctypes.c_void_p)), "eb_geometry_copy")
        return flag, vfrac, apx, apy, (fl.begin[0], fl.begin[1])

    def fill_ghosts(self, time, stream=None):
        check(self.lib.ocfd_level_fill_ghosts(self.h, time, _stream_ptr(stream)), "fill_ghosts")

