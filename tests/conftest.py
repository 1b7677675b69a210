import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libcudasirecon.so")


def pytest_collection_modifyitems(config, items):
    # keep the CPU suite runnable anywhere: gpu tests are skipped when no GPU is visible
    try:
        import ctypes
        ctypes.CDLL("libcuda.so.1")
        have_gpu = True
    except OSError:
        have_gpu = False
    if have_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA driver / GPU on this host")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)
