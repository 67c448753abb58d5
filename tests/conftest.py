import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")
    config.addinivalue_line("markers", "slow: longer oracle runs")


@pytest.fixture(scope="session")
def built_library():
    """Builds (incrementally) and loads libgansu_gb300.so."""
    from dft_gansu_gb300 import build as b
    b.build()
    from dft_gansu_gb300 import _capi
    return _capi.lib()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    return torch
