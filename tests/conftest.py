"""Test configuration: the `gpu` marker, import paths and shared helpers.

CPU tests (-m "not gpu") cover the oracle against its invariants and the committed
golden vectors, the host logic and the C ABI's exports. GPU tests call the CUDA
path through the C ABI and compare it with the oracle on the same inputs.
"""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "p2de.jl_gb300"))
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run on a GB300)")


def relerr(a, b, floor=0.0):
    """Normwise relative error ||a - b||_inf / max(||b||_inf, floor)."""
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), floor))


def has_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False
