import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a engine)")
    config.addinivalue_line("markers", "slow: minutes of oracle time (still part of the -m gpu run)")


@pytest.fixture(scope="session")
def o64():
    from oracle import Oracle
    return Oracle("f64")


@pytest.fixture(scope="session")
def o32():
    from oracle import Oracle
    return Oracle("f32")
