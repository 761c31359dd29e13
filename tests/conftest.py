import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(autouse=True)
def _bounds_checked_library(request):
    """With DFCSR_GB300_CHECKED=1 the package loads the bounds-checked
    library; every GPU test then also fails if one of its kernels recorded
    an out-of-range index (the checked library skips such an access and
    keeps the first failure's site and index)."""
    checked = os.environ.get("DFCSR_GB300_CHECKED", "") == "1"
    gpu = request.node.get_closest_marker("gpu") is not None
    if not (checked and gpu):
        yield
        return
    import torch
    if not torch.cuda.is_available():
        yield
        return
    from pydfcsr_gb300 import _lib
    assert _lib.load().dfcsr_bounds_checked() == 1
    _lib.bounds_status(reset=True)
    yield
    failure = _lib.bounds_status(reset=True)
    assert failure is None, f"index check failed in {request.node.nodeid}: (site, index) = {failure}"
