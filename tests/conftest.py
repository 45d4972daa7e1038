import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


def _have_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    """Skips (on CPU-only machines) unless a GPU is present; builds the library."""
    if not _have_gpu():
        pytest.skip("no CUDA device")
    from porescale_gb300 import _build
    _build.build_all()
    import porescale_gb300
    porescale_gb300.library()
    return True


@pytest.fixture(scope="session")
def oracle_lib():
    from porescale_gb300 import _build
    _build.build_oracle()
    import oracle
    oracle.lib()
    return oracle
