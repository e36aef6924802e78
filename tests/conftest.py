"""Test configuration: markers and import paths.

``gpu`` marks tests that need a CUDA device (they call libmmdg.so through its C ABI);
everything else runs on the CPU: the oracle against the reference's golden vectors,
host-side logic, and the C-ABI symbol table.
"""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "mcmurchie-davidson_gb300")
GOLDEN = os.path.join(REPO, "tests", "golden")
for p in (REPO, PKG, os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmmdg.so")


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    def load(name):
        return dict(np.load(os.path.join(GOLDEN, name), allow_pickle=False))
    return load


@pytest.fixture(scope="session")
def built_lib():
    """Build libmmdg.so (sm_103a, cross-compiled without a GPU) if needed."""
    sys.path.insert(0, PKG)
    import build as _b
    return _b.build()
