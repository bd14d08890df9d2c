import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Native build (no-op when up to date)."""
    from gpuexplore_gb300 import build
    build.build_all()
    return build


@pytest.fixture(scope="session")
def gpu(built):
    """The library on a GPU; the CUDA path must load and find a device.  Every
    run of the GPU tests computes the visited-set hash (off by default in the
    library), which the tests compare with the oracle's."""
    from gpuexplore_gb300 import lib
    lib.load()
    lib.DEFAULT_OPTIONS["set_hash"] = 1
    if lib.device_info(0) is None:
        pytest.fail("no CUDA device visible to libgpx")
    return lib
