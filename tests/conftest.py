import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the built library")


@pytest.fixture(scope="session")
def ctx():
    import corr_gb300

    c = corr_gb300.Context(0)
    yield c
    c.close()
