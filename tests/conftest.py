import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "joinproject-dim3_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def golden():
    import json

    import numpy as np

    d = os.path.join(ROOT, "tests", "golden")
    index = json.load(open(os.path.join(d, "golden_index.json")))
    arrays = np.load(os.path.join(d, "golden_arrays.npz"))
    return index, arrays


@pytest.fixture(scope="session")
def built():
    """Native libraries built in-tree (CUDA library, generators, oracle)."""
    import build as pkg_build

    from oracle import oracle_py

    pkg_build.build()
    oracle_py.build()
    return True


@pytest.fixture(scope="session")
def ctx(built):
    import dim3gpu

    c = dim3gpu.Context(0)
    yield c
    c.close()
