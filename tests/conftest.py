import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
for p in (REPO / "particle-life-app_gb300", REPO / "oracle", REPO / "tests", REPO):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA library)")


@pytest.fixture(scope="session")
def oracle():
    import orc

    orc.build()
    return orc


@pytest.fixture(scope="session")
def lib():
    """The CUDA library, loaded (built first if missing)."""
    from plgpu import _lib

    return _lib.load()


@pytest.fixture(scope="session")
def gpu():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    torch.cuda.init()
    return torch.device("cuda:0")
