import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library")


@pytest.fixture(scope="session")
def built():
    """Builds the CUDA library and the oracle once per session."""
    import __graft_entry__
    __graft_entry__.build()
    return True


def interior(a):
    return a[1:-1, 1:-1, 1:-1]


def rel_l2(a, b):
    a, b = interior(a), interior(b)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)
