import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    def load(name):
        return np.load(os.path.join(GOLDEN, name))
    return load


@pytest.fixture(autouse=True)
def _no_out_of_range_access(request):
    """With the bounds-checked library (ANL_DEBUG_LIB=1, python -m anneal_gb300.build --debug)
    every GPU test ends with no global access caught out of range by the kernels' checks."""
    yield
    if request.node.get_closest_marker("gpu") is None:
        return
    from anneal_gb300 import _native as N
    if not N.DEBUG_LIB:
        return
    import ctypes
    count, first = ctypes.c_longlong(0), (ctypes.c_longlong * 3)()
    N.check(N.load().anl_debug_oob(ctypes.byref(count), first), "anl_debug_oob")
    assert count.value == 0, (f"{count.value} out-of-range accesses; first: index {first[0]}, extent {first[1]}, "
                              f"source line {first[2]}")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O
