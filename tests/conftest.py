import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgdb")


def _cuda_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def ctx():
    """One library context for the GPU tests (fails loudly without libgdb)."""
    if not _cuda_available():
        pytest.skip("no CUDA device")
    from gpu_discovery_barrier_gb300 import gdb

    c = gdb.Ctx()
    yield c
    c.close()
