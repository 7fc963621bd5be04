import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, GOLDEN):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the sm_103a kernels")


@pytest.fixture(scope="session", autouse=True)
def built_library():
    """Builds libspn_su2.so and the oracle once per session (no-op when up to date)."""
    import __graft_entry__

    __graft_entry__.build()
    return True


# Normwise errors that the full-size parity tests measure, printed at the end of the run (also
# with -q) so that a run's log states them.
PARITY_REPORT: list[str] = []


def pytest_terminal_summary(terminalreporter):
    if PARITY_REPORT:
        terminalreporter.section("parity errors (normwise, GPU vs oracle)")
        for line in PARITY_REPORT:
            terminalreporter.write_line(line)
