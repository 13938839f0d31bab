import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT / "lapis-silo_gb300", ROOT / "oracle", ROOT / "tests", ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    """Builds librhygpu.so (sm_103a) and the CPU oracle once per session."""
    import build as pkg_build
    import oracle

    pkg_build.build()
    oracle.build()
    import rhydb_gpu

    rhydb_gpu.lib()
    yield


@pytest.fixture(scope="session")
def gpu_available():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False
