import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built native library")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def native_lib():
    from paraprobe_gb300 import build
    build.build()
    from paraprobe_gb300 import native
    return native.load()


@pytest.fixture(scope="session")
def ctx(native_lib):
    if not _has_gpu():
        pytest.skip("no CUDA device")
    from paraprobe_gb300 import native
    c = native.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O
