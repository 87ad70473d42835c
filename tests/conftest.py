import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

GOLDEN = os.path.join(ROOT, "tests", "golden")
SCENES = os.path.join(GOLDEN, "scenes")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA kernels through the C ABI")


@pytest.fixture(scope="session", autouse=True)
def built():
    """Builds the library and the oracle once per session (no-op when current)."""
    from mypbr_gb300 import build
    build.build()
    build.build_oracle()
    return True


def scene_path(name):
    return os.path.join(SCENES, name)


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
