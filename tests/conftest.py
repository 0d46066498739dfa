import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def _cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _cuda_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device in this process")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def sdlib():
    """The built C-ABI library (built on first use)."""
    from stardust_gb300 import build as sd_build
    sd_build.build()
    import stardust_gb300
    stardust_gb300.lib()
    return stardust_gb300


@pytest.fixture(scope="session")
def orc():
    """The CPU oracle (built on first use)."""
    from oracle import build as ob
    ob.build()
    from oracle import oracle
    oracle.lib()
    return oracle
