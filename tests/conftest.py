import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the sm_103a kernels")
    config.addinivalue_line("markers", "slow: long cases (the 512^3 benchmark domain); on the CPU they run only with "
                                       "SCORE_SLOW_TESTS=1, on the GPU always")


def pytest_collection_modifyitems(config, items):
    """CPU cases marked slow (minutes of single-threaded oracle work) run only on request;
    GPU cases marked slow take seconds on the device and always run."""
    if os.environ.get("SCORE_SLOW_TESTS") == "1":
        return
    skip = pytest.mark.skip(reason="slow CPU case: set SCORE_SLOW_TESTS=1 to run it")
    for item in items:
        if "slow" in item.keywords and "gpu" not in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def built():
    """Compile the native library and the oracle once per session."""
    import __graft_entry__
    __graft_entry__.build()
    return True


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu(built):
    if not has_gpu():
        pytest.fail("GPU test selected but no CUDA device is visible")
    return True


@pytest.fixture
def tmp_uds(tmp_path):
    def make(spec):
        return spec.write(tmp_path / "params.uds")
    return make
