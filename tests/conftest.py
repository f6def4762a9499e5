import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: full-size workloads")


@pytest.fixture(scope="session")
def gpu():
    """One decoding context for the GPU tests (the library must be built: __graft_entry__.build())."""
    from gpuzip_gb300 import gpuinflate

    g = gpuinflate.Gpu(0)
    yield g
    g.close()


@pytest.fixture(scope="session")
def gpu_small_segments():
    """A context with tiny segments: many segment boundaries per stream (16 KiB in, 8 MiB out)."""
    from gpuzip_gb300 import gpuinflate

    g = gpuinflate.Gpu(0, segment_out_mb=8, segment_in_kb=16)
    yield g
    g.close()
