import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")
    config.addinivalue_line("markers", "slow: long-running CPU statistics")


@pytest.fixture(scope="session")
def engine():
    """One propagator context for the whole GPU session (built in-tree first)."""
    from ismc_gb300 import build, Engine
    build.build()
    e = Engine(0)
    yield e
    e.close()
