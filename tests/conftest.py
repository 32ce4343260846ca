import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libstab_gb300.so")


@pytest.fixture(scope="session")
def ctx():
    """One library context on cuda:0 for the GPU tests."""
    import stab_gb300
    c = stab_gb300.Context(0)
    yield c
    c.close()
