import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the built CUDA library")


@pytest.fixture(scope="session")
def pkg():
    """The package, with libtebd_gb300.so built for this machine (no CPU fallback)."""
    import __graft_entry__ as ge

    ge._build_module().build()
    return ge.load_package()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.lib()
    return O


def gpu_present():
    try:
        import ctypes

        rt = ctypes.CDLL("libcudart.so")
    except OSError:
        try:
            import glob
            import ctypes

            c = sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*"))
            if not c:
                return False
            rt = ctypes.CDLL(c[0])
        except OSError:
            return False
    n = ctypes.c_int(0)
    return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
