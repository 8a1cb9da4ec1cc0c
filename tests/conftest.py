import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (str(ROOT / "ngia-metax_gb300"), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the native library, the oracle and (here) the reference makeDB once per session."""
    import __graft_entry__

    __graft_entry__.build()
    yield


@pytest.fixture(scope="session")
def cuda_device():
    import ngia

    if ngia.device_count() < 1:
        pytest.skip("no CUDA device")
    return 0
