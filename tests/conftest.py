import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run on the GB300)")


def _cuda():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _cuda():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def built():
    """Builds (or reuses) the GPU library and the oracle."""
    import __graft_entry__

    __graft_entry__.build()
    return True


@pytest.fixture(scope="session")
def ref_lib():
    """The reference shim compiled from rmagine's own sources, when present."""
    import ctypes

    from oracle import build_ref

    path = build_ref.build()
    if path is None or not Path(path).exists():
        pytest.skip("reference shim not built (rmagine checkout absent)")
    return ctypes.CDLL(str(path))
