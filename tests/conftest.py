"""Shared pytest setup.

Markers: ``gpu`` for tests that need a CUDA device (run with ``-m gpu`` on a
GB300); everything else runs on the CPU.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "oracle"), os.path.join(ROOT, "opencfd-amr_gb300"),
          os.path.join(ROOT, "tests"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def ref():
    from oracle import RefOracle, build_ref, reference_dir
    if reference_dir() is None:
        pytest.skip("reference sources not present on this machine")
    build_ref()
    return RefOracle()


@pytest.fixture(scope="session")
def oracle_omp():
    """The oracle's OpenMP build (bit-identical to the serial one: the threads
    split independent cells), for the runs at the configurations' sizes."""
    from oracle import Oracle
    return Oracle(openmp=True)


def golden(name):
    import numpy as np
    with np.load(os.path.join(ROOT, "tests", "golden", name + ".npz")) as f:
        return {k: f[k] for k in f.files}
