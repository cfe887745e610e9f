import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libsmac_gb300.so")


def gpu_available() -> bool:
    """True when the CUDA driver reports at least one device (no torch import needed)."""
    import ctypes
    try:
        cu = ctypes.CDLL("libcuda.so.1")
    except OSError:
        return False
    n = ctypes.c_int(0)
    return cu.cuInit(0) == 0 and cu.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0


@pytest.fixture(scope="session")
def cuda_lib():
    """The built CUDA library; GPU tests fail loudly if it cannot be built or loaded."""
    if not gpu_available():
        pytest.skip("no CUDA device")
    from minismac_gb300 import build, solver
    build.build()
    return solver.lib()


@pytest.fixture(scope="session")
def grid119():
    from minismac_gb300 import inputs
    return inputs.naca4_cgrid(119, 31)
