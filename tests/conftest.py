import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running parity case")


def gpu_available() -> bool:
    try:
        from adc_ottawa_gb300._native import lib
        import ctypes as C

        h = C.c_void_p()
        st = lib().adcgpu_ctx_create(0, C.byref(h))
        if st == 0:
            lib().adcgpu_ctx_destroy(h)
            return True
    except Exception:
        return False
    return False


@pytest.fixture(scope="session")
def built():
    import __graft_entry__ as g

    g.build()
    return True


@pytest.fixture(scope="session")
def gpu(built):
    if not gpu_available():
        pytest.fail("GPU test requested but no CUDA device could be opened")
    return True


_systems = {}


def system(no, nv, seed):
    """Seeded synthetic system (e, packed ERIs), cached per session."""
    key = (no, nv, seed)
    if key not in _systems:
        from adc_ottawa_gb300 import synth_system

        _systems[key] = synth_system(no, nv, seed)
    return _systems[key]


def sorted_coo(h, oi, oj):
    k = np.lexsort((oj, oi))
    return h[k], oi[k], oj[k]
