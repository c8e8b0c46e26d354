"""Python access to the ocfd C ABI (include/ocfd/ocfd.h).

The product is libocfd.so: hand-written sm_103a kernels behind a C ABI, with
the level driver (box tables, ghost fill, RK stages, graph capture) in C++ in
the same library.  This package only binds that ABI with ctypes so tests and
the benchmark can drive it with device buffers owned by PyTorch; there is no
computational fallback here - a call without the library or without a GPU
raises.
"""
from ._abi import (Array4, Box, Flag4, OcfdError, Parm, array4, box, flag4, lib, load,  # noqa: F401
                   status_string, check)
from .context import Context  # noqa: F401

NUM_GROW = 4
NCONS = 5
NSPEC = 9

VISC = 1
REDISTRIBUTE = 2
FLUX_FP32 = 4
PER_BOX = 8
GRAVITY = 16


def set_tma_staging(on):
    """Stage the FP32-flux form's tiles of depth >= 4 by TMA (the default) or with
    plain loads, in stage tables built from now on (a test hook: both give the
    same results)."""
    load().ocfd_set_tma_staging(1 if on else 0)
