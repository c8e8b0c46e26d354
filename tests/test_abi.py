"""The C-ABI library on a machine without a GPU: it builds, loads, exports every
symbol include/ocfd/*.h declares, its host-only parts agree with the oracle, and
its device entry points fail loudly instead of falling back to the CPU."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "ocfd", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        src = re.sub(r"#define[^\n]*", "", src)
        names |= set(re.findall(r"\b(ocfd_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


@pytest.fixture(scope="module")
def L():
    import ocfd
    return ocfd.load()


def test_exports_every_declared_symbol(L):
    names = declared_symbols()
    assert len(names) >= 8
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_built_for_sm103(L):
    assert L.ocfd_built_arch() == 1030
    assert L.ocfd_version() >= 1


def test_parm_default_matches_oracle(L, oracle):
    import ocfd
    from ocfd.context import default_parm
    p = default_parm()
    for f in ocfd.Parm.SCALARS:
        assert getattr(p, f) == getattr(oracle.parm, f), f
    o = oracle.parm
    assert [p.mw[i] for i in range(9)] == list(o.mw)
    lo = ["H2_lo", "O2_lo", "H2O_lo", "H_lo", "O_lo", "OH_lo", "HO2_lo", "H2O2_lo", "N2_lo"]
    for n, name in enumerate(lo):
        assert [getattr(p, name)[c] for c in range(7)] == list(o.nasa_lo[n])
        assert [getattr(p, name.replace("_lo", "_hi"))[c] for c in range(7)] == list(o.nasa_hi[n])
    assert [p.HP[i] for i in range(9)] == list(o.HP)
    assert [p.A0[i] for i in range(9)] == list(o.A0)
    assert [p.visccoeff[i] for i in range(45)] == list(o.visccoeff)
    assert [p.conductcoeff[i] for i in range(45)] == list(o.conductcoeff)
    assert [p.diffcoeff[i] for i in range(225)] == list(o.diffcoeff)


def test_parm_layout_matches_reference_order():
    # Source/Constants.H:9-60 member order, CHEM build: 16 doubles then 24 pointers
    import ocfd
    assert ctypes.sizeof(ocfd.Parm) == 16 * 8 + 24 * 8
    assert ocfd.Parm.eos_gamma.offset == 0 and ocfd.Parm.oneSix.offset == 15 * 8
    assert ocfd.Parm.mw.offset == 16 * 8 and ocfd.Parm.diffcoeff.offset == 39 * 8
    # amrex::Array4<double>: p, 3 x Long strides, Dim3 begin, Dim3 end, int ncomp
    assert ctypes.sizeof(ocfd.Array4) == 64
    assert ocfd.Array4.begin.offset == 32 and ocfd.Array4.end.offset == 44 and ocfd.Array4.ncomp.offset == 56


def test_status_strings(L):
    assert L.ocfd_status_string(0) == b"ok"
    assert L.ocfd_status_string(6) == b"no suitable device"


def test_no_device_fails_loudly(L):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import ocfd
    with pytest.raises(ocfd.OcfdError) as e:
        ocfd.Context()
    assert e.value.status == 6


def test_negative_floor_rejected(L):
    """The density / pressure floors must be >= 0 (the kernels compare against
    them on the integer bits): checked before any device work, so on any host."""
    import ocfd
    from ocfd.context import default_parm
    for field in ("smallr", "smallp"):
        p = default_parm()
        setattr(p, field, -1e-10)
        with pytest.raises(ocfd.OcfdError) as e:
            ocfd.Context(parm=p)
        assert e.value.status == 1, field  # OCFD_BAD_ARG
