import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgmorpho_gb300.so")


@pytest.fixture(scope="session")
def gm_ctx():
    from broxy_gb300 import api
    ctx = api.Context(0)
    yield ctx
    ctx.close_ctx()
