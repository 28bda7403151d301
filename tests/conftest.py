"""Test configuration: the ``gpu`` marker and shared fixtures.

``-m "not gpu"`` runs the CPU suite (oracle vs the golden fixtures, host-side
logic, library exports); ``-m gpu`` runs the parity tests, which call the CUDA
kernels through the C-ABI and need a GPU.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (parity tests through the C-ABI)")


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
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name)))
