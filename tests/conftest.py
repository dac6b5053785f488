import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 host)")


@pytest.fixture(scope="session", autouse=True)
def _oracle_built():
    """The CPU oracle is a few C files; build it if it is missing."""
    from cuminlp_gb300 import build
    build.build_oracle()
    yield


def bits_equal(a, b) -> bool:
    """Bit equality of two float arrays, treating +0 and -0 as equal and
    NaN equal to NaN."""
    import numpy as np
    a = np.asarray(a)
    b = np.asarray(b)
    if a.shape != b.shape:
        return False
    both_nan = np.isnan(a) & np.isnan(b)
    zero = (a == 0) & (b == 0)
    same = a.view(np.uint64 if a.dtype == np.float64 else np.uint32) == \
        b.view(np.uint64 if b.dtype == np.float64 else np.uint32)
    return bool(np.all(same | zero | both_nan))
