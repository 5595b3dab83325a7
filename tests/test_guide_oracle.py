"""The guiding network's CPU oracle (oracle/guide_oracle.py) checked on its
own: analytic gradients against central finite differences in float64, and
the vMF pieces against direct integration."""
import numpy as np

import guide_oracle as go


def random_params(seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(go.N_PARAMS)
    p[go.W1:go.B1] = rng.uniform(-0.2, 0.2, go.B1 - go.W1)
    p[go.B1:go.W2] = rng.uniform(-0.1, 0.1, 64)
    p[go.W2:go.B2] = rng.uniform(-0.3, 0.3, 64 * 64)
    p[go.B2:go.W3] = rng.uniform(-0.1, 0.1, 64)
    p[go.W3:go.W3 + 40 * 64] = rng.uniform(-0.3, 0.3, 40 * 64)
    p[go.B3:go.B3 + 40] = rng.uniform(-0.5, 0.5, 40)
    return p


def random_records(n, seed):
    rng = np.random.default_rng(seed)
    rec = np.zeros((n, 12))
    rec[:, 0:3] = rng.uniform(0, 1, (n, 3))
    nrm = rng.normal(size=(n, 3))
    rec[:, 3:6] = nrm / np.linalg.norm(nrm, axis=1, keepdims=True)
    w = rng.normal(size=(n, 3))
    rec[:, 6:9] = w / np.linalg.norm(w, axis=1, keepdims=True)
    rec[:, 9] = rng.uniform(0.05, 2.0, n)
    rec[:, 10] = rng.uniform(0.0, 3.0, n)
    return rec


def test_gradient_matches_finite_differences():
    p = random_params(1)
    rec = random_records(12, 2)
    loss, g = go.gradient(p, rec, fp16=False)
    rng = np.random.default_rng(3)
    idx = np.concatenate([rng.choice(np.arange(go.W1, go.B1), 12), rng.choice(np.arange(go.B1, go.W2), 4),
                          rng.choice(np.arange(go.W2, go.B2), 12), rng.choice(np.arange(go.B2, go.W3), 4),
                          rng.choice(np.arange(go.W3, go.W3 + 40 * 64), 16), np.arange(go.B3, go.B3 + 40)])
    h = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += h
        lp, _ = go.gradient(q, rec, fp16=False)
        q[i] -= 2 * h
        lm, _ = go.gradient(q, rec, fp16=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(fd)) + 1e-7, (i, fd, g[i])


def test_vmf_lobe_integrates_to_one_and_samples_follow_it():
    rng = np.random.default_rng(4)
    w = rng.normal(size=(400000, 3))
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    for kappa in (0.01, 1.0, 20.0):
        mu = np.array([[0.0, 0.6, 0.8]])
        p = go.vmf_pdf(np.repeat(mu, len(w), 0), np.full(len(w), kappa), w)
        assert abs(p.mean() * 4 * np.pi - 1.0) < 0.02
        s = go.sample_vmf(np.repeat(mu, 200000, 0), np.full(200000, kappa), rng.uniform(size=200000),
                          rng.uniform(size=200000))
        # mean cosine to mu: coth(k) - 1/k
        want = 1 / np.tanh(kappa) - 1 / kappa
        assert abs((s @ mu[0]).mean() - want) < 0.01
