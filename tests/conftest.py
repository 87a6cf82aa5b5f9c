import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


@pytest.fixture(scope="session")
def lib():
    """The native library, built in-tree if missing (nvcc cross-compiles without a GPU)."""
    import __graft_entry__ as g
    so = os.path.join(ROOT, "jax-fem_gb300", "libjaxfem_gb300.so")
    if not os.path.exists(so):
        g.build()
    import jax_fem_gb300 as jf
    return jf._lib.load()


@pytest.fixture(scope="session")
def cuda(lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def golden(name):
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))
