import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built libbonsai_gpu.so")


@pytest.fixture(scope="session")
def gpu_ctx():
    from bonsai_gb300 import gpu
    ctx = gpu.Context(0)
    yield ctx
    ctx.close()
