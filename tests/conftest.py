import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) device")


@pytest.fixture(scope="session")
def engine():
    import twochnrg_gb300 as tg
    e = tg.Engine(0)
    yield e
    e.close()
