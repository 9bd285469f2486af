"""The CPU oracle of the learned proposal, checked on its own (no GPU):
the vMF mixture is a density on the sphere, and the loss gradient of the
float64 autograd path agrees with finite differences."""
import numpy as np
import pytest

import learned_ref as L

torch = pytest.importorskip("torch")


def test_vmf_mixture_integrates_to_one():
    rng = np.random.default_rng(0)
    raw = rng.normal(size=(1, 40))
    raw[0, 4::5] = rng.uniform(-3, 5, 8)  # a spread of concentrations
    d = rng.normal(size=(400_000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    integral = L.vmf_pdf(np.repeat(raw, len(d), 0), d).mean() * 4 * np.pi
    assert abs(integral - 1) < 5e-3


def test_loss_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    params = L.init_params(2).astype(np.float64)
    params[-40:] = rng.normal(size=40) * 0.3
    n = 64
    bbox = np.array([-1.0, -1.0, -1.0, 1.0, 1.0, 1.0])
    pos = rng.uniform(-1, 1, (n, 3))
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    w = rng.lognormal(size=n)
    f = L.encode(pos, nrm, bbox)
    loss, g = L.loss_and_grads(params, f, d, w)
    for idx in rng.choice(len(params), 12, replace=False):
        e = np.zeros_like(params)
        e[idx] = 1e-6
        lp, _ = L.loss_and_grads(params + e, f, d, w)
        lm, _ = L.loss_and_grads(params - e, f, d, w)
        fd = (lp - lm) / 2e-6
        assert abs(fd - g[idx]) <= 1e-5 + 1e-4 * abs(fd), (idx, fd, g[idx])
