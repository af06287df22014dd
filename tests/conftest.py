import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if stale) and load libphgpu.so; fails loudly when it cannot be built."""
    from phasta_gb300 import build
    build.build()
    from phasta_gb300 import _lib
    return _lib.lib()
