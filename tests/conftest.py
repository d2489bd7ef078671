import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
if str(ROOT / "tests") not in sys.path:
    sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA library)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build libdem_gb300 (nvcc cross-compiles without a GPU) and the oracle once."""
    from gpucode_gb300 import build

    build.build()
    import _harness

    if not _harness.ORACLE_LIB.exists() or \
            _harness.ORACLE_LIB.stat().st_mtime < (_harness.ORACLE_DIR / "dem_oracle.c").stat().st_mtime:
        _harness.build_oracle()
    yield


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def cuda():
    if not gpu_available():
        pytest.fail("a gpu-marked test ran without a CUDA device")
    import torch

    torch.cuda.init()
    return torch.device("cuda:0")
