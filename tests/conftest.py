import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (a GB300)")
    config.addinivalue_line("markers", "slow: long-running parity case")


# where CPU tests look for the reference's core/ sources (read-only); tests
# that need them skip themselves when they are absent
REFERENCE_CORE = os.environ.get("FLUID2D_CORE", "/root/reference/core")


def reference_core(marker="fluid2d.py"):
    """The reference's core/ directory, or skip the calling test."""
    if not os.path.exists(os.path.join(REFERENCE_CORE, marker)):
        pytest.skip("reference sources not present")
    return REFERENCE_CORE


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if gpu_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device here")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)
