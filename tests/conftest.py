import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "oracle", ROOT / "tests" / "golden", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine")


@pytest.fixture(scope="session")
def engine_lib():
    """Build (if needed) and load libfwgb.so."""
    from fullwave25_gb300 import build, engine

    build.build()
    return engine.load_library()


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected but no CUDA device is visible")
    return torch
