import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:  # pragma: no cover
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def oracle():
    from oracle import fri_oracle
    fri_oracle.build()
    fri_oracle.lib()
    return fri_oracle


@pytest.fixture(scope="session")
def gpulib():
    """The CUDA library, built in-tree if needed; fails loudly if it cannot load."""
    from fricc_gb300 import build as b
    from fricc_gb300 import _lib
    b.build()
    return _lib.load()


def golden(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name))
