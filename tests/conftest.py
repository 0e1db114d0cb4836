import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (str(ROOT / "cellspe-tasklib_gb300"), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _cuda_ok() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def cg():
    """The engine's C ABI.  GPU tests fail loudly if the library is missing."""
    import cellspe_gpu

    if not _cuda_ok():
        pytest.skip("no CUDA device")
    cellspe_gpu.lib()
    return cellspe_gpu


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.lib()
    return oracle
