import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def engine_lib():
    from axicor_gb300 import build as B
    B.build()
    from axicor_gb300 import _native
    return _native.lib()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    return oracle.lib()


def _gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu(engine_lib):
    """Skips nothing: a gpu-marked test on a machine without a GPU fails loudly."""
    if not _gpu_available():
        pytest.fail("this test needs a CUDA GPU")
    return engine_lib
