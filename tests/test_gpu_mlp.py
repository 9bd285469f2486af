"""The learned proposal's network on the tensor cores against the CPU oracle."""
import numpy as np
import pytest

import learned_ref as L
import pppm_gb300 as P

pytestmark = pytest.mark.gpu


def _inputs(n, seed):
    rng = np.random.default_rng(seed)
    bbox = np.array([-30.0, -10.5, -30.0, 30.0, 10.5, 30.0])
    pos = (bbox[:3] + rng.uniform(size=(n, 3)) * (bbox[3:] - bbox[:3])).astype(np.float32)
    nrm = rng.normal(size=(n, 3))
    nrm = (nrm / np.linalg.norm(nrm, axis=1, keepdims=True)).astype(np.float32)
    return pos, nrm, bbox


@pytest.mark.parametrize("n", [1, 1000, 300_001])
def test_mlp_forward_matches_oracle(ctx, n):
    pos, nrm, bbox = _inputs(n, 5)
    params = L.init_params(3)
    params[-40:] = np.random.default_rng(4).normal(size=40).astype(np.float32) * 0.1  # nonzero output bias
    out = ctx.mlp_forward(params, pos, nrm, bbox)
    feats = L.encode(pos, nrm, bbox)
    ref = L.forward(params, feats, fp16=True)
    scale = np.abs(ref).mean()
    err = np.abs(out - ref)
    # FP16 activations may round differently where the FP32 sums differ in
    # the last bits: allow rare one-ulp FP16 flips, bound them tightly overall
    assert np.quantile(err, 0.999) <= 2e-3 * scale + 1e-3 * np.abs(ref).max() * 0, (err.max(), scale)
    assert err.max() <= 3e-2 * scale + 1e-2 * np.abs(ref).max()
    # against the exact FP64 network: the FP16 error stays at the 1e-2 level
    exact = L.forward(params, feats, fp16=False)
    rel = np.abs(out - exact).mean() / np.abs(exact).mean()
    assert rel < 2e-2, rel


@pytest.mark.parametrize("n", [1000, 70_000])
def test_mlp_grad_matches_oracle(ctx, n):
    """Loss and parameter gradient of the tensor-core training kernel against
    float64 autograd on the CPU (the GPU keeps FP16 weights and activations,
    so the comparison is at the 1e-2 level)."""
    pos, nrm, bbox = _inputs(n, 7)
    rng = np.random.default_rng(8)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    w = rng.lognormal(0.0, 1.0, n)
    w[rng.uniform(size=n) < 0.1] = 0.0  # zero-weight records contribute nothing
    params = L.init_params(11)
    params[-40:] = rng.normal(size=40).astype(np.float32) * 0.5
    rec = np.concatenate([pos, nrm, d, w[:, None]], 1).astype(np.float32)
    loss, g = ctx.mlp_grad(params, rec, bbox)
    feats = L.encode(pos, nrm, bbox)
    ref_loss, ref_g = L.loss_and_grads(params, feats, rec[:, 6:9].astype(np.float64), rec[:, 9].astype(np.float64))
    assert abs(loss - ref_loss) <= 1e-2 * abs(ref_loss), (loss, ref_loss)
    cos = float(g @ ref_g / (np.linalg.norm(g) * np.linalg.norm(ref_g)))
    rel = float(np.linalg.norm(g - ref_g) / np.linalg.norm(ref_g))
    print(f"n={n}: loss {loss:.6f} vs {ref_loss:.6f}, grad cos {cos:.6f}, rel {rel:.3e}")
    assert cos > 0.999, cos
    assert rel < 5e-2, rel
