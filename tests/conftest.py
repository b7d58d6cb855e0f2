import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("oracle", "gevolution-1.2_gb300"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def oracle():
    import gevoracle
    gevoracle.lib()
    return gevoracle


@pytest.fixture(scope="session")
def gpu():
    import gev_gb300
    gev_gb300.lib()
    return gev_gb300


def golden(name):
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", name), allow_pickle=False)
