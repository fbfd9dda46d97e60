import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.dirname(os.path.abspath(__file__))
for p in (REPO, HERE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgvom_gb300.so")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if needed) and load the CUDA library; fail loudly without it."""
    from gvom_gb300 import build, _lib
    build.build()
    return _lib.load()


GOLDEN = os.path.join(HERE, "golden")


def golden_files():
    """The mapper scene fixtures (ros_*.npz hold the ROS node's payloads and
    morph_*.npz the 2-D image kernels' outputs instead)."""
    return sorted(f for f in os.listdir(GOLDEN) if f.endswith(".npz") and not f.startswith(("ros_", "morph_")))
