import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def built_library():
    """Build the C-ABI library if it is missing or stale, then load it."""
    from optika_gb300 import _lib, build

    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def cuda(built_library):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    torch.cuda.set_device(0)
    return torch.device("cuda", 0)
