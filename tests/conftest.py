import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")


def _has_gpu():
    return os.path.exists("/dev/nvidiactl") or os.path.exists("/dev/nvidia0")


def pytest_collection_modifyitems(config, items):
    # On a machine without an NVIDIA device the GPU tests cannot run; when one is
    # present they always run (and fail loudly if the extension is missing).
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no NVIDIA device on this machine")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)
