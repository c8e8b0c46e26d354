"""Reacting level binding (ocfd_react_* in include/ocfd/ocfd.h): multispecies
flow with operator-split Li-Dryer chemistry, one CUDA graph per step."""
from __future__ import annotations

import ctypes

import numpy as np

from ._abi import Box, check, declare, load
from .context import _stream_ptr
from .level import EbDesc, Level, LevelDesc

NCOMP = 14
_vp = ctypes.c_void_p


class ReactDesc(ctypes.Structure):
    _fields_ = [("level", LevelDesc), ("rk_order", ctypes.c_int32), ("chem_substeps", ctypes.c_int32),
                ("dt", ctypes.c_double), ("flags", ctypes.c_uint32), ("binned_chem", ctypes.c_int32)]


declare("ocfd_react_create", ctypes.c_int, [_vp, ctypes.POINTER(ReactDesc), ctypes.POINTER(_vp)])
declare("ocfd_react_destroy", ctypes.c_int, [_vp])
declare("ocfd_react_level", _vp, [_vp])
declare("ocfd_react_advance", ctypes.c_int, [_vp, ctypes.c_int, _vp])
declare("ocfd_react_launches_per_step", ctypes.c_int, [_vp])
declare("ocfd_react_profile_chem", ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_double), _vp])
declare("ocfd_react_set_eb", ctypes.c_int, [_vp, ctypes.POINTER(EbDesc)])
declare("ocfd_react_box_classes", ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int32)])
declare("ocfd_chem_state_tpx", ctypes.c_int, [_vp, ctypes.c_int64, _vp, _vp, _vp, _vp, _vp, _vp])


class Reactor:
    def __init__(self, ctx, boxes, domain_hi, dx, lo_bc=(0, 0, 0), hi_bc=(0, 0, 0), dt=1e-8, rk_order=2,
                 chem_substeps=4, visc=True, binned=False, prob_lo=(0.0, 0.0, 0.0), flux_fp32=False):
        self.ctx = ctx
        self.lib = load()
        d = ReactDesc()
        bx = (Box * len(boxes))()
        for i, (lo, hi) in enumerate(boxes):
            bx[i].lo[:] = list(lo)
            bx[i].hi[:] = list(hi)
        d.level.nbox = len(boxes)
        d.level.boxes = bx
        d.level.domain.lo[:] = [0, 0, 0]
        d.level.domain.hi[:] = list(domain_hi)
        d.level.lo_bc[:] = list(lo_bc)
        d.level.hi_bc[:] = list(hi_bc)
        d.level.dx[:] = list(dx)
        d.level.prob_lo[:] = list(prob_lo)
        d.level.tile = -1
        d.rk_order = rk_order
        d.chem_substeps = chem_substeps
        d.dt = dt
        d.flags = (1 if visc else 0) | (4 if flux_fp32 else 0)
        d.binned_chem = 1 if binned else 0
        self._keep = bx
        h = ctypes.c_void_p()
        check(self.lib.ocfd_react_create(ctx.h, ctypes.byref(d), ctypes.byref(h)), "ocfd_react_create")
        self.h = h
        self.level = Level.wrap(ctx, self.lib.ocfd_react_level(h), boxes, (0, 0, 0), domain_hi, ncomp=NCOMP)

    def close(self):
        if self.h:
            self.lib.ocfd_react_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def advance(self, nsteps, stream=None):
        check(self.lib.ocfd_react_advance(self.h, nsteps, _stream_ptr(stream)), "ocfd_react_advance")

    def set_eb(self, desc):
        """Cut the level with an embedded body (ocfd.level.eb_desc(...))."""
        check(self.lib.ocfd_react_set_eb(self.h, ctypes.byref(desc)), "ocfd_react_set_eb")

    def box_classes(self):
        out = (ctypes.c_int32 * len(self.level.boxes))()
        check(self.lib.ocfd_react_box_classes(self.h, out), "ocfd_react_box_classes")
        return list(out)

    def launches_per_step(self):
        return int(self.lib.ocfd_react_launches_per_step(self.h))

    def profile_chem(self, reps=5, stream=None):
        ms = ctypes.c_double()
        check(self.lib.ocfd_react_profile_chem(self.h, reps, ctypes.byref(ms), _stream_ptr(stream)), "profile_chem")
        return ms.value


def state_tpx(ctx, T, p, X):
    """Conserved state (14, ...) of resting mixtures at T, p (arrays of one
    shape) with mole fractions X (9, ...), computed on the GPU."""
    import torch
    shape = np.shape(T)
    n = int(np.prod(shape))
    dev = torch.device("cuda")
    Tt = torch.as_tensor(np.ascontiguousarray(T, dtype=np.float64).ravel(), device=dev)
    pt = torch.as_tensor(np.array(np.broadcast_to(p, shape), dtype=np.float64).ravel(), device=dev)
    Xt = torch.as_tensor(np.ascontiguousarray(np.asarray(X, dtype=np.float64).reshape(9, n)), device=dev)
    U = torch.empty((5, n), dtype=torch.float64, device=dev)
    R = torch.empty((9, n), dtype=torch.float64, device=dev)
    check(load().ocfd_chem_state_tpx(ctx.h, n, _vp(Tt.data_ptr()), _vp(pt.data_ptr()), _vp(Xt.data_ptr()),
                                     _vp(U.data_ptr()), _vp(R.data_ptr()), _stream_ptr(None)), "ocfd_chem_state_tpx")
    torch.cuda.synchronize()
    return np.concatenate([U.cpu().numpy(), R.cpu().numpy()]).reshape((14,) + tuple(shape))
