import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds libmbg.so, the CLI and the oracle library once if any is missing."""
    import oracle
    import upmabossg_gb300 as mbg
    from upmabossg_gb300 import build as b

    if not (os.path.exists(mbg.LIB_PATH) and os.path.exists(mbg.CLI_PATH)):
        b.build()
    if not os.path.exists(oracle.LIB):
        oracle.build()
    yield


@pytest.fixture(scope="session")
def has_gpu():
    import upmabossg_gb300 as mbg

    return mbg.device_count() > 0
