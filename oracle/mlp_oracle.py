"""CPU restatement of the cost-model network (uxxxxxxxxh_gb300/csrc/mlp.cu).

TEST INFRASTRUCTURE ONLY: the checker the GPU forward pass and gradients are
compared against.  float64 numpy, same parameter layout (per layer
[W (out x in), b (out)]), ReLU between layers, loss = mean((p - y)^2)."""
from __future__ import annotations

import numpy as np


def unpack(w: np.ndarray, dims: list) -> list:
    layers, o = [], 0
    for din, dout in zip(dims[:-1], dims[1:]):
        W = w[o:o + din * dout].reshape(dout, din)
        o += din * dout
        b = w[o:o + dout]
        o += dout
        layers.append((W, b))
    return layers


def forward(w, dims, x):
    acts = [np.asarray(x, np.float64)]
    L = len(dims) - 1
    for l, (W, b) in enumerate(unpack(np.asarray(w, np.float64), dims)):
        z = acts[-1] @ W.T + b
        acts.append(np.maximum(z, 0.0) if l + 1 < L else z)
    return acts


def loss_grad(w, dims, x, y):
    acts = forward(w, dims, x)
    n = x.shape[0]
    p = acts[-1][:, 0]
    loss = float(np.mean((p - y) ** 2))
    d = (2.0 * (p - y) / n)[:, None]
    grads = []
    layers = unpack(np.asarray(w, np.float64), dims)
    L = len(layers)
    for l in range(L - 1, -1, -1):
        W, b = layers[l]
        if l + 1 < L:
            d = d * (acts[l + 1] > 0)
        grads.append((d.T @ acts[l], d.sum(axis=0)))
        d = d @ W
    flat = []
    for dW, db in reversed(grads):
        flat.append(dW.reshape(-1))
        flat.append(db)
    return loss, np.concatenate(flat)
