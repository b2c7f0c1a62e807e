import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


# (case, tally z-scores) recorded by the statistical parity tests; printed in
# the terminal summary so that every run shows the per-tally agreement
PARITY_Z = []


def pytest_terminal_summary(terminalreporter):
    if not PARITY_Z:
        return
    names = ("A", "R_d", "R_s", "T_d", "T_u")
    tr = terminalreporter
    tr.write_sep("-", "per-tally z = (GPU - reference) / combined standard error")
    tr.write_line(f"{'case':34s} " + " ".join(f"{n:>7s}" for n in names) + "   max|z|")
    for case, z in PARITY_Z:
        tr.write_line(f"{case:34s} " + " ".join(f"{x:+7.2f}" for x in z) +
                      f"   {max(abs(x) for x in z):6.2f}")


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
