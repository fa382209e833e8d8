"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
from __future__ import annotations

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build(ref=False)
    return oracle.Oracle()


@pytest.fixture(scope="session")
def reference():
    import oracle
    if not oracle.Reference.available():
        if oracle.ref_src() is not None:
            oracle.build(ref=True)
        else:
            pytest.skip("reference library not built and GD_REFERENCE_SRC not set")
    return oracle.Reference()


@pytest.fixture(scope="session")
def gdlib():
    """The CUDA library, built for sm_103a (nvcc cross-compiles without a GPU)."""
    from golikov_2d_gb300 import _build
    _build.build()
    import golikov_2d_gb300 as g
    return g.load()


@pytest.fixture(scope="session")
def cuda():
    """A CUDA device; GPU tests fail loudly if the library cannot be built or loaded."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from golikov_2d_gb300 import _build
    _build.build()
    import golikov_2d_gb300 as g
    g.load()
    return torch.device("cuda:0")


def golden(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name))
