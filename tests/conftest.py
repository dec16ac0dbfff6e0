"""Shared test set-up.  GPU tests carry @pytest.mark.gpu and run only on a
machine with a GB300; everything else runs on the CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle32():
    from oracle import build
    build.build_oracle()
    from oracle.pyoracle import Oracle
    return Oracle("f32")


@pytest.fixture(scope="session")
def oracle64():
    from oracle import build
    build.build_oracle()
    from oracle.pyoracle import Oracle
    return Oracle("f64")


def golden(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name))
