"""Shared helpers for the test suite."""
import numpy as np


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def relmax(a, b, region=None):
    """max |a-b| / max |b| over a region (tuple of slices)."""
    if region is not None:
        a, b = a[region], b[region]
    den = float(np.max(np.abs(b)))
    if den == 0.0:
        den = 1.0
    return float(np.max(np.abs(a - b))) / den


def interior_rows(ny):
    """rows 1..ny (the reference leaves y-ghost rows stale in places)."""
    return (slice(None), slice(1, ny + 1), slice(None))
