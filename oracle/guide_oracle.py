"""CPU restatement of the learned guiding proposal (network, vMF mixture,
loss and its gradient, Adam) in numpy.

TEST INFRASTRUCTURE ONLY: the oracle the tests compare the GPU kernels of
drawlab_gb300/csrc/guide.{cuh,cu} against.  The network has no counterpart in the
reference (its guiding code is absent); this file states the model the GPU
implements, in float64, with the GPU's fp16 rounding points emulated where
asked (`fp16=True`): weights, encodings and hidden activations are fp16,
accumulations and the output layer are wide.
"""
from __future__ import annotations

import numpy as np

N_IN, N_FREQ, N_ENC, N_HID, N_LOBES, N_OUT, N_OUT_PAD = 6, 12, 144, 64, 8, 40, 48
W1, B1 = 0, 64 * 144
W2, B2 = B1 + 64, B1 + 64 + 64 * 64
W3 = B2 + 64
B3 = W3 + 48 * 64
N_PARAMS = B3 + 48
LOGK_MIN, LOGK_MAX = -3.0, 8.0


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[W1:B1].reshape(64, 144), p[B1:W2], p[W2:B2].reshape(64, 64), p[B2:W3],
            p[W3:B3].reshape(48, 64), p[B3:B3 + 48])


def pack(w1, b1, w2, b2, w3, b3):
    return np.concatenate([w1.ravel(), b1, w2.ravel(), b2, w3.ravel(), b3]).astype(np.float64)


def _h(x, fp16):
    return x.astype(np.float16).astype(np.float64) if fp16 else x


def encode(inp, fp16=True):
    """inp (n, 6) -> (n, 144): per scalar, (sin, cos)(2^(k-3) pi x) for k < 12."""
    inp = np.asarray(inp, np.float64)
    k = (2.0 ** (np.arange(N_FREQ) - 3)) * np.pi
    a = inp[:, :, None] * k[None, None, :]                     # (n, 6, 12)
    e = np.stack([np.sin(a), np.cos(a)], axis=-1).reshape(len(inp), N_ENC)
    return _h(e, fp16)


def forward(params, inp, fp16=True):
    w1, b1, w2, b2, w3, b3 = unpack(params)
    w1, w2, w3 = _h(w1, fp16), _h(w2, fp16), _h(w3, fp16)
    x = encode(inp, fp16)
    h1 = _h(np.maximum(x @ w1.T + b1, 0.0), fp16)
    h2 = _h(np.maximum(h1 @ w2.T + b2, 0.0), fp16)
    o = h2 @ w3.T + b3
    return o[:, :N_OUT], (x, h1, h2, w1, w2, w3)


def decode(o):
    """(n, 40) -> mu (n, 8, 3), kappa (n, 8), lambda (n, 8), inv_len, clamped."""
    o = o.reshape(-1, N_LOBES, 5)
    m = o[..., :3]
    ln = np.linalg.norm(m, axis=-1)
    ok = ln > 1e-6
    mu = np.where(ok[..., None], m / np.where(ok, ln, 1.0)[..., None], np.array([0.0, 0.0, 1.0]))
    inv_len = np.where(ok, 1.0 / np.where(ok, ln, 1.0), 0.0)
    lk = o[..., 3]
    clamped = (lk < LOGK_MIN) | (lk > LOGK_MAX)
    kappa = np.exp(np.clip(lk, LOGK_MIN, LOGK_MAX))
    z = o[..., 4] - o[..., 4].max(axis=-1, keepdims=True)
    lam = np.exp(z) / np.exp(z).sum(axis=-1, keepdims=True)
    return mu, kappa, lam, inv_len, clamped


def vmf_pdf(mu, kappa, w):
    d = (mu * w[..., None, :]).sum(-1) if w.ndim == mu.ndim - 1 else (mu * w).sum(-1)
    small = kappa < 1e-4
    k = np.where(small, 1.0, kappa)
    p = k / (2 * np.pi * (-np.expm1(-2 * k))) * np.exp(k * (d - 1))
    return np.where(small, 0.25 / np.pi, p)


def mixture_pdf(o, w):
    mu, kappa, lam, _, _ = decode(o)
    return (lam * vmf_pdf(mu, kappa, np.asarray(w, np.float64))).sum(-1)


CLAMP = 20.0


def loss_and_dout(o, rec):
    """Loss of records `rec` (n, 12) and dLoss/do (n, 40) for outputs o.
    Record weights L/p are normalised by their batch mean and clamped at
    CLAMP times it."""
    n = len(rec)
    L, pdf, w = rec[:, 10], rec[:, 9], rec[:, 6:9]
    ratio = np.where(pdf > 0, L / np.where(pdf > 0, pdf, 1.0), 0.0)
    mean = np.float32(np.float32(ratio.astype(np.float32).sum()) / np.float32(n)) if n else 0.0
    scale = np.where((pdf > 0) & (mean > 0), np.minimum(ratio / mean if mean > 0 else 0.0, CLAMP) / n, 0.0)
    mu, kappa, lam, inv_len, clamped = decode(o)
    pj = lam * vmf_pdf(mu, kappa, w)
    q = pj.sum(-1)
    good = (q > 1e-30) & (scale > 0)
    qs = np.where(good, q, 1.0)
    r = pj / qs[:, None]
    dot = (mu * w[:, None, :]).sum(-1)
    s = scale[:, None]
    d = np.zeros((n, N_LOBES, 5))
    d[..., 4] = -s * (r - lam)
    k = kappa
    t = np.where(k < 1e-4, 0.0, 1.0 - 2.0 * k / np.expm1(2.0 * np.where(k < 1e-4, 1.0, k)) + k * (dot - 1.0))
    d[..., 3] = np.where(clamped, 0.0, -s * r * t)
    f = -s * r * k * inv_len
    d[..., :3] = f[..., None] * (w[:, None, :] - dot[..., None] * mu)
    d[~good] = 0.0
    loss = np.where(good, -scale * np.log(qs), 0.0).sum()
    return loss, d.reshape(n, N_OUT)


def gradient(params, rec, fp16=True):
    """(loss, gradient) of the batch loss with the GPU's rounding points."""
    rec = np.asarray(rec, np.float64)
    o, (x, h1, h2, w1, w2, w3) = forward(params, rec[:, :6], fp16)
    loss, dout = loss_and_dout(o, rec)
    d0 = np.zeros((len(rec), N_OUT_PAD))
    d0[:, :N_OUT] = dout
    # activation gradients are rounded to fp16 loss-scaled: times n (so that
    # they stay out of fp16's subnormal range), saturated at +-65504
    S = float(len(rec))

    def hs(x):
        return _h(np.clip(x * S, -65504.0, 65504.0), fp16) / S if fp16 else x

    d0h = hs(d0)
    d2 = (d0h @ w3) * (h2 > 0)
    d2h = hs(d2)
    d1 = (d2h @ w2) * (h1 > 0)
    d1h = hs(d1)
    # bias gradients: sums of the rounded activation gradients, as the GPU
    # forms them (a product with a column of ones)
    g_b3, g_b2, g_b1 = d0h.sum(0), d2h.sum(0), d1h.sum(0)
    g_w3 = d0h.T @ h2
    g_w2 = d2h.T @ h1
    g_w1 = d1h.T @ x
    g_w3[N_OUT:] = 0.0
    g_b3[N_OUT:] = 0.0
    return loss, pack(g_w1, g_b1, g_w2, g_b2, g_w3, g_b3)


def adam(params, grad, m, v, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (step counts from 1); padding rows of layer 3 stay 0."""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    p = params - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    p[W3 + N_OUT * 64:B3] = 0.0
    p[B3 + N_OUT:] = 0.0
    return p, m, v


def sample_vmf(mu, kappa, u1, u2):
    """Directions from single vMF lobes (mu (n, 3), kappa (n,))."""
    w = np.where(kappa < 1e-4, 2 * u1 - 1,
                 1 + np.log(u1 + (1 - u1) * np.exp(-2 * kappa)) / np.where(kappa < 1e-4, 1.0, kappa))
    w = np.clip(w, -1, 1)
    v = np.sqrt(np.maximum(0, 1 - w * w))
    phi = 2 * np.pi * u2
    a = np.where(np.abs(mu[:, 0:1]) > 0.9, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    t = np.cross(mu, a)
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    b = np.cross(mu, t)
    return v[:, None] * (np.cos(phi)[:, None] * t + np.sin(phi)[:, None] * b) + w[:, None] * mu
