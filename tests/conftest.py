import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libfhist")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


def torch_ordered_context(device: int = 0):
    """A library Context whose raw entry-point calls start after the work torch
    has queued: the tests make their device buffers on torch's stream, and the
    library runs on a stream of its own."""
    import torch
    from theses_code_gb300._lib import Context

    class TorchOrdered(Context):
        def call(self, name, *args):
            torch.cuda.synchronize()
            return super().call(name, *args)

    return TorchOrdered(device)
