import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300)")


def _cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def built_lib():
    """Build (if stale) and return the engine library path."""
    from gpusort_gb300 import _build
    return _build.build()


@pytest.fixture(scope="session")
def ctx(built_lib):
    """One engine context on cuda:0 on torch's current stream."""
    if not _cuda_available():
        pytest.fail("GPU test collected without a CUDA device")
    import torch
    from gpusort_gb300 import Context
    torch.cuda.init()
    c = Context(0)
    c.set_stream(torch.cuda.current_stream().cuda_stream)
    yield c
    c.close()
