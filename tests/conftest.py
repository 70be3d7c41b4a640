import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: full-size workloads")


@pytest.fixture(scope="session")
def built_lib():
    """Builds libconvgpu.so in-tree (no-op when up to date) and loads it."""
    from convfpga_gb300 import build, load_library

    build.build()
    return load_library()


@pytest.fixture(scope="session")
def gpu(built_lib):
    """Initialised library on cuda:0 for GPU tests."""
    import convfpga_gb300 as cg

    rc = cg.fpga_initialize("cuda:0", "convgpu_plans.json", False)
    assert rc == 0, cg.last_error()
    yield cg
