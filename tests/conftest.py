import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(REPO, "vegas-rs_gb300"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def V():
    import vegas_gb300

    vegas_gb300.lib()
    return vegas_gb300


@pytest.fixture(scope="session")
def O():
    import oracle

    oracle.lib()
    return oracle
