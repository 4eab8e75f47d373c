import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built extension")


def golden(name):
    import numpy as np
    return np.load(os.path.join(REPO, "tests", "golden", name))


@pytest.fixture(scope="session")
def gold():
    return golden
