import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def tb():
    import tight_binding_gb300 as tb
    return tb


@pytest.fixture(scope="session")
def gpu(tb):
    if tb.device_count() < 1:
        pytest.fail("GPU test run without a visible CUDA device")
    return tb
