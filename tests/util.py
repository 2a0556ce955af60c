import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


def relerr(a, b):
    """max |a - b| relative to the largest magnitude of b (field-wise scale)."""
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    assert a.shape == b.shape, (a.shape, b.shape)
    if a.size == 0:
        return 0.0
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)
