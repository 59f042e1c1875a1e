import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 (sm_103a) device")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds (incrementally) the CUDA library and the CPU oracle once."""
    from kagayaki_gb300 import build as kb
    kb.build()
    from oracle import orc
    orc.build()
    yield


def golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


C1_LO, C1_HI = (-4.99, 0.01, -4.99), (4.99, 9.99, 4.99)
