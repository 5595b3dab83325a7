"""The guiding network on the GPU (tensor-core forward / backward kernels)
against the CPU oracle (oracle/guide_oracle.py, with the GPU's fp16
rounding points): outputs, loss, gradients and one Adam step; and training
that fits a known directional distribution."""
import numpy as np
import pytest

import guide_oracle as go
from drawlab_gb300 import api
from test_guide_oracle import random_params, random_records

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return api.Context(0)


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


@pytest.mark.parametrize("n", [1, 37, 128, 1000, 100000])
def test_forward_matches_oracle(ctx, n):
    """tcgen05 inference (128-row tiles; a ragged last tile, many tiles per
    block) against the oracle."""
    g = api.Guide(ctx)
    p = random_params(5).astype(np.float32)
    g.set_params(p)
    np.testing.assert_array_equal(g.params(), p)
    inp = random_records(n, 6)[:, :6]
    out = g.forward(inp)
    want, _ = go.forward(p.astype(np.float64), inp, fp16=True)
    # fp16 activations: agreement to fp16-accumulation level
    assert rel(out, want) < 2e-3, rel(out, want)
    np.testing.assert_allclose(out, want, atol=2e-2 * np.abs(want).max())


@pytest.mark.parametrize("n", [1000, 16384, 37, 100000])
def test_gradient_matches_oracle(ctx, n):
    """Loss and gradients against the oracle: 37 records fill part of one
    tile (the weight-gradient products then sum padding records, whose
    gradients are zero); 1000 and 16384 records give each training block
    one tile; 100000 records give a block five or six tiles (the two
    encoding buffers alternate, the gradient sums accumulate in tensor
    memory), whose partial sums the reduction adds."""
    g = api.Guide(ctx)
    p = random_params(7).astype(np.float32)
    g.set_params(p)
    rec = random_records(n, 8)
    loss, grad = g.gradient(rec)
    wl, wg = go.gradient(p.astype(np.float64), rec.astype(np.float32).astype(np.float64), fp16=True)
    assert abs(loss - wl) <= 1e-3 * abs(wl), (loss, wl)
    for name, a, b in [("W1", go.W1, go.B1), ("b1", go.B1, go.W2), ("W2", go.W2, go.B2), ("b2", go.B2, go.W3),
                       ("W3", go.W3, go.B3), ("b3", go.B3, go.N_PARAMS)]:
        e = rel(grad[a:b], wg[a:b])
        assert e < 1e-2, (name, e)


def test_adam_step_matches_oracle(ctx):
    g = api.Guide(ctx, learning_rate=1e-3)
    p = random_params(9).astype(np.float32)
    g.set_params(p)
    rec = random_records(4096, 10)
    _, grad = g.gradient(rec)
    g.train(rec, steps=1)
    got = g.params().astype(np.float64)
    want, _, _ = go.adam(p.astype(np.float64), grad.astype(np.float64), np.zeros(go.N_PARAMS),
                         np.zeros(go.N_PARAMS), 1, lr=1e-3)
    close = np.abs(got - want) <= 1e-6 + 1e-6 * np.abs(want)
    assert close.mean() > 0.999, close.mean()
    assert np.all(got[go.W3 + 40 * 64:go.B3] == 0) and np.all(got[go.B3 + 40:] == 0)


def target_records(n, rng):
    """Incident radiance proportional to a position-dependent vMF lobe:
    directions uniform on the sphere (pdf 1/4pi), L = the lobe's density."""
    rec = np.zeros((n, 12), np.float32)
    pos = rng.uniform(0, 1, (n, 3))
    rec[:, 0:3] = pos
    rec[:, 5] = 1.0                        # normal +z everywhere
    w = rng.normal(size=(n, 3))
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    rec[:, 6:9] = w
    rec[:, 9] = 1.0 / (4 * np.pi)
    mu = target_mu(pos)
    rec[:, 10] = go.vmf_pdf(mu[:, None, :], np.full((n, 1), 30.0), w)[:, 0]
    return rec


def target_mu(pos):
    a = np.pi * pos[:, 0]                  # the lobe turns with x
    mu = np.stack([np.cos(a), np.zeros_like(a), np.sin(a)], axis=1)
    return mu


def test_training_fits_a_known_distribution(ctx):
    g = api.Guide(ctx, learning_rate=3e-3, seed=3)
    rng = np.random.default_rng(11)
    test = target_records(2048, np.random.default_rng(12))
    l0, _ = g.gradient(test)
    for it in range(300):
        g.train(target_records(16384, rng), steps=1)
    l1, _ = g.gradient(test)
    assert l1 < l0 - 1.0, (l0, l1)
    # the learned mixture puts far more density at the target lobe's mean
    # than at the opposite direction
    pos = np.random.default_rng(13).uniform(0, 1, (256, 3))
    inp = np.zeros((256, 6), np.float32)
    inp[:, :3] = pos
    inp[:, 5] = 1.0
    out = g.forward(inp).astype(np.float64)
    mu = target_mu(pos)
    q_at = go.mixture_pdf(out, mu)
    q_opp = go.mixture_pdf(out, -mu)
    assert np.median(q_at / q_opp) > 20, np.median(q_at / q_opp)
    assert np.median(q_at) > 1.0          # a uniform sphere would give 0.08
