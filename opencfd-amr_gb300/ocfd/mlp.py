"""Chemistry surrogate network binding (ocfd_mlp_* in include/ocfd/ocfd.h):
BF16 tensor-core (tcgen05) forward, backward and Adam kernels."""
from __future__ import annotations

import ctypes

import numpy as np

from ._abi import check, declare, load
from .context import _stream_ptr

WTOT, BTOT = 53248, 528
_vp = ctypes.c_void_p
_fp = ctypes.POINTER(ctypes.c_float)
declare("ocfd_mlp_create", ctypes.c_int, [_vp, ctypes.c_int32, ctypes.c_uint64, ctypes.POINTER(_vp)])
declare("ocfd_mlp_destroy", ctypes.c_int, [_vp])
declare("ocfd_mlp_set_norm", ctypes.c_int, [_vp, _fp, _fp, _fp, _fp])
declare("ocfd_mlp_get_params", ctypes.c_int, [_vp, _vp, _vp])
declare("ocfd_mlp_set_target_scale", ctypes.c_int, [_vp, _fp])
declare("ocfd_mlp_set_params", ctypes.c_int, [_vp, _vp, _vp])
declare("ocfd_mlp_forward", ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int64, _vp])
declare("ocfd_mlp_train_step", ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int64, ctypes.c_float, ctypes.c_int32,
                                              _fp, _vp, _vp, _vp])


def _f(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(_fp)


class Mlp:
    def __init__(self, ctx, max_batch=8192, seed=1):
        self.ctx = ctx
        self.lib = load()
        h = ctypes.c_void_p()
        check(self.lib.ocfd_mlp_create(ctx.h, max_batch, seed, ctypes.byref(h)), "ocfd_mlp_create")
        self.h = h
        self.max_batch = max_batch

    def close(self):
        if self.h:
            self.lib.ocfd_mlp_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_norm(self, in_mu, in_isd, out_mu, out_sd):
        a = [_f(x) for x in (in_mu, in_isd, out_mu, out_sd)]
        check(self.lib.ocfd_mlp_set_norm(self.h, *[p for _, p in a]), "ocfd_mlp_set_norm")

    def set_target_scale(self, scale):
        a, p = _f(scale)
        check(self.lib.ocfd_mlp_set_target_scale(self.h, p), "ocfd_mlp_set_target_scale")

    def get_params(self):
        W = np.zeros(WTOT, np.float32)
        b = np.zeros(BTOT, np.float32)
        check(self.lib.ocfd_mlp_get_params(self.h, W.ctypes.data, b.ctypes.data), "ocfd_mlp_get_params")
        return W, b

    def set_params(self, W, b):
        W = np.ascontiguousarray(W, np.float32)
        b = np.ascontiguousarray(b, np.float32)
        check(self.lib.ocfd_mlp_set_params(self.h, W.ctypes.data, b.ctypes.data), "ocfd_mlp_set_params")

    def forward(self, X, stream=None):
        """X: CUDA float32 tensor [M x 12] (normalised); returns [M x 10]."""
        import torch
        Y = torch.empty((X.shape[0], 10), dtype=torch.float32, device=X.device)
        check(self.lib.ocfd_mlp_forward(self.h, X.data_ptr(), Y.data_ptr(), X.shape[0], _stream_ptr(stream)),
              "ocfd_mlp_forward")
        return Y

    def train_step(self, X, T, lr=1e-3, update=True, grads=False, stream=None):
        loss = ctypes.c_float()
        gW = np.zeros(WTOT, np.float32) if grads else None
        gb = np.zeros(BTOT, np.float32) if grads else None
        check(self.lib.ocfd_mlp_train_step(self.h, X.data_ptr(), T.data_ptr(), X.shape[0], lr, int(update),
                                           ctypes.byref(loss), gW.ctypes.data if grads else None,
                                           gb.ctypes.data if grads else None, _stream_ptr(stream)),
              "ocfd_mlp_train_step")
        return loss.value, gW, gb
