import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture
def tile_path(monkeypatch):
    """The per-step tile passes for every window (FWI_CLUSTER=0): tests of properties the tile
    passes hold between storage modes, launch groupings and graph replay, which the small-shot
    cluster path (one launch per phase, full storage only, another summation order) does not
    share bit for bit."""
    monkeypatch.setenv("FWI_CLUSTER", "0")
    yield
