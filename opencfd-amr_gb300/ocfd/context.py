"""Context object and per-box calls of the C ABI (host-side mirror of the
reference's per-box RHS interface, Source/Advance.cpp:182-418)."""
from __future__ import annotations

import ctypes

from ._abi import Array4, Parm, array4, box, check, flag4, load


def _stream_ptr(stream):
    if stream is None:
        import torch
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if isinstance(stream, int):
        return ctypes.c_void_p(stream)
    return ctypes.c_void_p(stream.cuda_stream)


def default_parm():
    p = Parm()
    check(load().ocfd_parm_default(ctypes.byref(p)), "ocfd_parm_default")
    return p


class Context:
    """Owns an ocfd_context (device tables, scratch pool, error word)."""

    def __init__(self, parm=None, device=0):
        L = load()
        self.parm = parm if parm is not None else default_parm()
        h = ctypes.c_void_p()
        check(L.ocfd_context_create(ctypes.byref(self.parm), device, ctypes.byref(h)),
              "ocfd_context_create")
        self.h = h
        self.lib = L

    def close(self):
        if self.h:
            self.lib.ocfd_context_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, stream=None):
        w = ctypes.c_uint32()
        check(self.lib.ocfd_context_check(self.h, _stream_ptr(stream), ctypes.byref(w)),
              "ocfd_context_check")
        return w.value

    # ---- per-box right-hand sides ------------------------------------------
    def rhs_regular_box(self, S, dSdt, lo, hi, dxinv, flags=0, flux=None, S_begin=None,
                        stream=None):
        """S: (>=5, nz+8, ny+8, nx+8) tensor beginning at lo-4 (or S_begin);
        dSdt: (>=5, nz, ny, nx) at lo; flux: None or three face tensors at lo."""
        sb = S_begin if S_begin is not None else tuple(l - 4 for l in lo)
        aS = array4(S, sb)
        aD = array4(dSdt, lo)
        fl = None
        if flux is not None:
            fl = (Array4 * 3)(*[array4(f, lo) for f in flux])
        dx = (ctypes.c_double * 3)(*dxinv)
        st = self.lib.ocfd_rhs_regular_box_f64(self.h, ctypes.byref(aS), ctypes.byref(aD), fl,
                                               box(lo, hi), dx, flags, _stream_ptr(stream))
        check(st, "ocfd_rhs_regular_box_f64")

    def rhs_eb_box(self, S, dSdt, geom, lo, hi, dxinv, flags=0, flux=None, S_begin=None,
                   stream=None):
        """Cut-cell box.  geom: dict of CUDA tensors flag (int32 view of the
        uint32 words, grown by 4), vfrac (grown by 4), apx, apy, apz (faces of
        the box)."""
        sb = S_begin if S_begin is not None else tuple(l - 4 for l in lo)
        g4 = tuple(l - 4 for l in lo)
        aS, aD = array4(S, sb), array4(dSdt, lo)
        fl = None
        if flux is not None:
            fl = (Array4 * 3)(*[array4(f, lo) for f in flux])
        af = flag4(geom["flag"], g4)
        av = array4(geom["vfrac"], g4)
        ap = [array4(geom[k], lo) for k in ("apx", "apy", "apz")]
        dx = (ctypes.c_double * 3)(*dxinv)
        st = self.lib.ocfd_rhs_eb_box_f64(self.h, ctypes.byref(aS), ctypes.byref(aD), fl,
                                          ctypes.byref(af), ctypes.byref(av), ctypes.byref(ap[0]),
                                          ctypes.byref(ap[1]), ctypes.byref(ap[2]), None, None,
                                          box(lo, hi), dx, flags, _stream_ptr(stream))
        check(st, "ocfd_rhs_eb_box_f64")

    # ---- chemistry ---------------------------------------------------------
    def chem_advance_box(self, S, spec, lo, hi, dt, S_begin=None, spec_begin=None, stream=None):
        """One chemistry substep in place on (5, nz, ny, nx) / (9, nz, ny, nx)
        tensors (or larger arrays described by *_begin)."""
        aS = array4(S, S_begin if S_begin is not None else lo)
        aR = array4(spec, spec_begin if spec_begin is not None else lo)
        check(self.lib.ocfd_chem_advance_box_f64(self.h, ctypes.byref(aS), ctypes.byref(aR),
                                                  box(lo, hi), dt, _stream_ptr(stream)),
              "ocfd_chem_advance_box_f64")

    def spec_renorm_box(self, S, spec, lo, hi, S_begin=None, spec_begin=None, stream=None):
        aS = array4(S, S_begin if S_begin is not None else lo)
        aR = array4(spec, spec_begin if spec_begin is not None else lo)
        check(self.lib.ocfd_spec_renorm_box_f64(self.h, ctypes.byref(aS), ctypes.byref(aR),
                                                 box(lo, hi), _stream_ptr(stream)),
              "ocfd_spec_renorm_box_f64")

    def rhs_chem_box(self, S, spec, dSdt, dSdt_spec, lo, hi, dxinv, flags=0, flux=None,
                     flux_spec=None, stream=None):
        """Regular multispecies box; S (5) and spec (9) grown by 4 around lo..hi."""
        g4 = tuple(l - 4 for l in lo)
        aS, aR = array4(S, g4), array4(spec, g4)
        aD, aDs = array4(dSdt, lo), array4(dSdt_spec, lo)
        fl = (Array4 * 3)(*[array4(f, lo) for f in flux]) if flux is not None else None
        fs = (Array4 * 3)(*[array4(f, lo) for f in flux_spec]) if flux_spec is not None else None
        dx = (ctypes.c_double * 3)(*dxinv)
        check(self.lib.ocfd_rhs_chem_box_f64(self.h, ctypes.byref(aS), ctypes.byref(aR),
                                              ctypes.byref(aD), ctypes.byref(aDs), fl, fs,
                                              box(lo, hi), dx, flags, _stream_ptr(stream)),
              "ocfd_rhs_chem_box_f64")

    def rhs_chem_eb_box(self, S, spec, dSdt, dSdt_spec, geom, lo, hi, dxinv, flags=0, flux=None,
                        flux_spec=None, stream=None):
        """Cut multispecies box; S, spec and geom flag/vfrac grown by 4 around lo..hi."""
        g4 = tuple(l - 4 for l in lo)
        aS, aR = array4(S, g4), array4(spec, g4)
        aD, aDs = array4(dSdt, lo), array4(dSdt_spec, lo)
        fl = (Array4 * 3)(*[array4(f, lo) for f in flux]) if flux is not None else None
        fs = (Array4 * 3)(*[array4(f, lo) for f in flux_spec]) if flux_spec is not None else None
        af, av = flag4(geom["flag"], g4), array4(geom["vfrac"], g4)
        ap = [array4(geom[k], lo) for k in ("apx", "apy", "apz")]
        dx = (ctypes.c_double * 3)(*dxinv)
        check(self.lib.ocfd_rhs_chem_eb_box_f64(self.h, ctypes.byref(aS), ctypes.byref(aR),
                                                 ctypes.byref(aD), ctypes.byref(aDs), fl, fs,
                                                 ctypes.byref(af), ctypes.byref(av), ctypes.byref(ap[0]),
                                                 ctypes.byref(ap[1]), ctypes.byref(ap[2]), None, None,
                                                 box(lo, hi), dx, flags, _stream_ptr(stream)),
              "ocfd_rhs_chem_eb_box_f64")
