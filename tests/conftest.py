import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


def _ensure_built():
    from mdet_gb300 import build as b
    from oracle import oracle

    b.build()
    if not os.path.exists(oracle.LIB):
        oracle.build()


_ensure_built()


@pytest.fixture(scope="session")
def gpu_ctx():
    import mdet_gb300 as m

    ctx = m.Context(0)
    yield ctx
    ctx.close()
