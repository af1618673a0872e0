import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libselfgpu.so")


@pytest.fixture(scope="session", autouse=True)
def _native_library():
    """Builds the product library in-tree once when it is missing (a fresh checkout): the CPU tests use its host-side
    set-up routines and its export table.  It is the library itself, not a fallback (there is none)."""
    from self_gb300 import _native as nat
    if not os.path.exists(nat.LIB_PATH):
        from self_gb300 import build as B
        B.build()
    yield


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def gpu_ctx():
    import self_gb300 as sg
    ctx = sg.Context(0)
    yield ctx
    ctx.close()
