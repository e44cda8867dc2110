import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the device kernels)")


@pytest.fixture(scope="session")
def ctx():
    import scirs_gb300 as S

    c = S.Context(0)
    yield c
    c.close()
