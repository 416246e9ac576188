import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "svt-jpeg-xs_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the product path")


@pytest.fixture(scope="session")
def oracle():
    import oracle_lib

    oracle_lib.build_oracle()
    return oracle_lib


@pytest.fixture(scope="session")
def jxs_lib():
    """The product library, built in-tree if needed."""
    import build as pkg_build

    pkg_build.build()
    import jxs

    jxs.lib()
    return jxs


@pytest.fixture(scope="session")
def gpu(jxs_lib):
    import ctypes

    n = ctypes.c_int()
    cudart = ctypes.CDLL(jxs_lib.LIB_PATH)
    if cudart.jxs_gpu_device_count() < 1:
        pytest.fail("a GPU test ran without a CUDA device")
    return jxs_lib
