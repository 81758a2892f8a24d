"""Helpers shared by the GPU parity tests."""
import numpy as np
import pytest


def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def rel_err(got, ref, floor_frac=1e-6):
    """max |got - ref| / max(|ref|, floor_frac * max|ref|) — the error statement of the path."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    floor = floor_frac * max(np.max(np.abs(ref)), 1e-300)
    return float(np.max(np.abs(got - ref) / np.maximum(np.abs(ref), floor)))
