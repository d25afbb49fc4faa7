import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libibmgpu.so")
    config.addinivalue_line("markers", "slow: longer CPU test")


def load_package():
    """The package directory name contains hyphens, so import it by name."""
    return importlib.import_module("ibm-3d-fpc_gb300")


@pytest.fixture(scope="session")
def ibm():
    return load_package()


@pytest.fixture(scope="session")
def pyoracle():
    import pyoracle as po
    return po


def gpu_available() -> bool:
    try:
        import torch  # noqa: F401  (only to ask the CUDA driver whether a GPU exists)
        return torch.cuda.is_available()
    except Exception:
        return False
