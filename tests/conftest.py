import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (parity tests through the C ABI)")


@pytest.fixture(scope="session")
def oracle():
    """The CPU restatement (built on first use)."""
    from oracle import pyoracle
    pyoracle.build(ref=False)
    return pyoracle.Oracle()


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    gdir = os.path.join(ROOT, "tests", "golden")

    def load(name):
        return np.load(os.path.join(gdir, name))
    return load
