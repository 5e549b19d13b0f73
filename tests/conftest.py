import os
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and libgkrt.so built for it")


@pytest.fixture(scope="session")
def gkrt_lib():
    """Path of the in-tree libgkrt.so (built on demand where nvcc exists)."""
    from gknextengine_gb300 import build, native
    if not os.path.exists(native.LIB_PATH):
        build.build()
    return native.LIB_PATH


@pytest.fixture(scope="session")
def renderer_factory(gkrt_lib):
    from gknextengine_gb300.renderer import PathTracingRenderer
    made = []

    def make():
        r = PathTracingRenderer(0)
        made.append(r)
        return r

    yield make
    for r in made:
        r.close()
