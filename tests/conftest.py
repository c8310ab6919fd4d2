import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgdft_xc.so")


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    def load(name):
        return np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))

    return load


@pytest.fixture(scope="session")
def built_lib():
    """Build libgdft_xc.so in-tree if needed (nvcc cross-compiles without a GPU)."""
    from graddft_gb300 import build

    return build.build()
