"""CPU reference of the surrogate MLP: TEST INFRASTRUCTURE ONLY.

numpy forward pass, softmax cross-entropy and backward pass of the ensemble member the device
trains (upmabossg_gb300/csrc/device/mlp.cu, csrc/host/surrogate.cpp): ReLU hidden layers, linear
output layer, mean cross-entropy against target distributions. With ``bf16=True`` the values the
device stores in BF16 (inputs, weights, hidden activations, output and hidden gradients) are
rounded to BF16 at the same places, and everything else is computed in float64, so the device's
gradients can be compared closely. Parameters are flattened per layer as W [in][out] row-major,
then b, like mbg_surrogate_get_params. The analytic gradient is itself checked by finite
differences in tests/test_oracle.py.
"""
from __future__ import annotations

import numpy as np


def bf16_round(a):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unflatten(params, dims):
    """Per-layer (W, b) from the flat parameter vector; dims = [in, hidden..., out]."""
    out, o = [], 0
    for i, j in zip(dims[:-1], dims[1:]):
        W = np.asarray(params[o:o + i * j], dtype=np.float64).reshape(i, j)
        o += i * j
        b = np.asarray(params[o:o + j], dtype=np.float64)
        o += j
        out.append((W, b))
    return out


def forward(params, dims, x, bf16=True):
    """Logits and the per-layer inputs (for the backward pass)."""
    rnd = bf16_round if bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    layers = unflatten(params, dims)
    a = rnd(x)
    inputs = []
    for li, (W, b) in enumerate(layers):
        inputs.append(a)
        z = a @ rnd(W) + b
        if li < len(layers) - 1:
            a = rnd(np.maximum(z, 0.0))
        else:
            return z, inputs


def softmax(z):
    z = z - z.max(axis=1, keepdims=True)
    e = np.exp(z)
    return e / e.sum(axis=1, keepdims=True)


def loss_and_grad(params, dims, x, y, bf16=True):
    """Mean cross-entropy and its gradient (flattened like the parameters)."""
    rnd = bf16_round if bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    layers = unflatten(params, dims)
    z, inputs = forward(params, dims, x, bf16)
    p = softmax(z)
    n = len(x)
    logp = z - z.max(axis=1, keepdims=True)
    logp = logp - np.log(np.exp(logp).sum(axis=1, keepdims=True))
    loss = float(-(np.asarray(y) * logp).sum() / n)
    d = rnd((p - y) / n)
    grads = [None] * len(layers)
    for li in range(len(layers) - 1, -1, -1):
        W, _ = layers[li]
        a_in = inputs[li]
        grads[li] = (a_in.T @ d, d.sum(axis=0))
        if li > 0:
            da = d @ rnd(W).T
            d = rnd(np.where(a_in > 0, da, 0.0))
    flat = np.concatenate([np.concatenate([g[0].ravel(), g[1]]) for g in grads])
    return loss, flat


def init_params(dims, rng):
    parts = []
    for li, (i, j) in enumerate(zip(dims[:-1], dims[1:])):
        sd = np.sqrt((1.0 if li == len(dims) - 2 else 2.0) / i)
        parts += [rng.normal(0, sd, i * j), np.zeros(j)]
    return np.concatenate(parts).astype(np.float32)
