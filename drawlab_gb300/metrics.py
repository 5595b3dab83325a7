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


def relmse_robust(img: np.ndarray, ref: np.ndarray, eps: float = 0.01, discard: float = 1e-3) -> float:
    """relMSE after discarding the largest `discard` fraction of per-pixel
    errors (fireflies: single samples that dominate the plain mean)."""
    img = np.asarray(img, np.float64)
    ref = np.asarray(ref, np.float64)
    if img.shape != ref.shape:
        raise ValueError("shape mismatch %s vs %s" % (img.shape, ref.shape))
    e = ((img - ref) ** 2 / (ref * ref + eps)).reshape(img.shape[0] * img.shape[1], -1).mean(axis=1)
    k = int(np.floor(len(e) * (1.0 - discard)))
    return float(np.sort(e)[:max(k, 1)].mean())
