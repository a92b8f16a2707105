import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


def gpu_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def port():
    import oracle

    return oracle.port()


@pytest.fixture(scope="session")
def ref():
    import oracle

    r = oracle.ref()
    if r is None:
        pytest.skip("reference sources not present: the compiled reference is unavailable")
    return r


@pytest.fixture(scope="session")
def gpu_ctx():
    # No skip: a GPU test without a usable device or library must fail loudly.
    from inmyroom_vulkan_gb300 import capi

    ctx = capi.Context()
    yield ctx
    ctx.close()
