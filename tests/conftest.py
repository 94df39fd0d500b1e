import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "fly-brain_gb300"), os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")
    config.addinivalue_line("markers", "slow: full-size workloads")


@pytest.fixture(scope="session")
def golden_cases():
    return sorted(f for f in os.listdir(GOLDEN) if f.endswith(".npz"))
