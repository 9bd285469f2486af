"""CPU oracle of the learned photon proposal (test infrastructure only).

The proposal has no counterpart in the reference renderer; this module
restates its definition from the formulas so the GPU kernels can be checked:
the input encoding, the 80-64-64-64-40 network (optionally emulating FP16
weights and activations with FP32 accumulation), the von Mises-Fisher mixture
the outputs parameterise, and the training loss with its gradients (torch
float64 autograd on the CPU).
"""
from __future__ import annotations

import numpy as np

FREQS = 12
LOBES = 8
SHAPES = [(64, 80), (64, 64), (64, 64), (40, 64)]
N_PARAMS = sum(o * i + o for o, i in SHAPES)


def unpack(params):
    """Flat parameters -> [(W[out][in], b[out])] * 4."""
    p = np.asarray(params).reshape(-1)
    out, k = [], 0
    for o, i in SHAPES:
        W = p[k:k + o * i].reshape(o, i)
        k += o * i
        b = p[k:k + o]
        k += o
        out.append((W, b))
    assert k == p.size
    return out


def init_params(seed):
    """He-style initialisation used by the renderer (seeded)."""
    rng = np.random.default_rng(seed)
    parts = []
    for o, i in SHAPES:
        parts.append((rng.standard_normal((o, i)) * np.sqrt(2.0 / i)).reshape(-1))
        parts.append(np.zeros(o))
    return np.concatenate(parts).astype(np.float32)


def encode(pos, nrm, bbox):
    """80 features per row, computed in float32 like the device: x = (p - o) * s
    per axis, then sin/cos(2^k pi x) for k < 12, the normal and five zeros."""
    pos = np.asarray(pos, np.float32)
    o = np.asarray(bbox[:3], np.float64).astype(np.float32)
    s = (1.0 / np.maximum(np.asarray(bbox[3:]) - np.asarray(bbox[:3]), 1e-12)).astype(np.float32)
    x = ((pos - o) * s).astype(np.float32)
    f = np.zeros((pos.shape[0], 80), np.float64)
    for a in range(3):
        t = x[:, a].astype(np.float64)
        for k in range(FREQS):
            f[:, a * 24 + 2 * k] = np.sin(np.pi * t)
            f[:, a * 24 + 2 * k + 1] = np.cos(np.pi * t)
            t = t * 2.0
    f[:, 72:75] = nrm
    return f


def forward(params, feats, fp16=True):
    """Raw 40 outputs. fp16=True rounds weights and inputs/activations of every
    layer to FP16 and accumulates in float32, as the tensor-core kernel does."""
    layers = unpack(params)
    a = np.asarray(feats, np.float64)
    for li, (W, b) in enumerate(layers):
        if fp16:
            a16 = a.astype(np.float16).astype(np.float32)
            W16 = np.asarray(W, np.float32).astype(np.float16).astype(np.float32)
            z = a16 @ W16.T + np.asarray(b, np.float32)
        else:
            z = a @ np.asarray(W, np.float64).T + b
        a = np.maximum(z, 0.0) if li < 3 else z
    return a


def mixture(raw):
    """(weights[8], means[8][3] unit, kappa[8]) from raw outputs (n x 40):
    softmax logits, normalised means, kappa = exp(clamp(log kappa, -4, 7))."""
    raw = np.asarray(raw, np.float64).reshape(-1, LOBES, 5)
    lg = raw[..., 0]
    w = np.exp(lg - lg.max(-1, keepdims=True))
    w /= w.sum(-1, keepdims=True)
    mu = raw[..., 1:4]
    mu = mu / np.maximum(np.linalg.norm(mu, axis=-1, keepdims=True), 1e-12)
    kappa = np.exp(np.clip(raw[..., 4], -4.0, 7.0))
    return w, mu, kappa


def vmf_pdf(raw, dirs):
    """Mixture density of unit directions dirs (n x 3) under raw outputs."""
    w, mu, k = mixture(raw)
    d = np.asarray(dirs, np.float64)[:, None, :]
    cosv = (mu * d).sum(-1)
    norm = k / (2.0 * np.pi * (1.0 - np.exp(-2.0 * k)))
    return (w * norm * np.exp(k * (cosv - 1.0))).sum(-1)


def loss_and_grads(params, feats, dirs, weights):
    """Weighted negative log-likelihood  sum_i w_i * -log q(d_i | x_i) / sum_i w_i
    and its gradient w.r.t. the flat parameters, in float64 autograd (no FP16
    emulation: the reference gradient)."""
    import torch

    p = torch.tensor(np.asarray(params, np.float64), requires_grad=True)
    x = torch.tensor(np.asarray(feats, np.float64))
    d = torch.tensor(np.asarray(dirs, np.float64))
    wt = torch.tensor(np.asarray(weights, np.float64))
    k = 0
    a = x
    for li, (o, i) in enumerate(SHAPES):
        W = p[k:k + o * i].view(o, i)
        k += o * i
        b = p[k:k + o]
        k += o
        a = a @ W.T + b
        if li < 3:
            a = torch.relu(a)
    raw = a.view(-1, LOBES, 5)
    logw = torch.log_softmax(raw[..., 0], -1)
    mu = raw[..., 1:4]
    mu = mu / torch.clamp(mu.norm(dim=-1, keepdim=True), min=1e-12)
    lk = torch.clamp(raw[..., 4], -4.0, 7.0)
    kap = torch.exp(lk)
    cosv = (mu * d[:, None, :]).sum(-1)
    lognorm = lk - np.log(2.0 * np.pi) - torch.log1p(-torch.exp(-2.0 * kap))
    logq = torch.logsumexp(logw + lognorm + kap * (cosv - 1.0), -1)
    loss = -(wt * logq).sum() / wt.sum()
    loss.backward()
    return float(loss.item()), p.grad.numpy().copy()
