"""Image error metrics for renderer comparisons."""
from __future__ import annotations

import numpy as np


def relmse(img: np.ndarray, ref: np.ndarray, eps: float = 0.01) -> float:
    """Relative mean squared error: mean over pixels and channels of
    (img - ref)^2 / (ref^2 + eps)."""
    img = np.asarray(img, np.float64)
    ref = np.asarray(ref, np.float64)
    if img.shape != ref.shape:
        raise ValueError("shape mismatch %s vs %s" % (img.shape, ref.shape))
    return float(np.mean((img - ref) ** 2 / (ref * ref + eps)))
