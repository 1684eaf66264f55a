import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built CUDA library")


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if needed) and load libsam_gpu.so; GPU tests fail loudly without it."""
    from sam_gb300 import build as B
    from sam_gb300 import sam_gpu
    B.build()
    return sam_gpu.load_library()
