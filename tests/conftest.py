import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if stale) and loads the in-tree CUDA library; the tests that
    use it must run where a GPU is present."""
    from puresoft3d_gb300 import pipeline
    return pipeline.library()
