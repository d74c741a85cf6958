"""CPU FP64 restatement of the warm-start MLP -- TEST INFRASTRUCTURE ONLY.

The network (16 -> 128 -> ReLU -> 128 -> ReLU -> 32) and its loss (BCE on the
10 passive-set logits + amp_weight * MSE of softplus(amplitude outputs)) are
the engine's own design with no counterpart in the reference, so this module
is the checker of the hand-written GPU kernels (test-regression_gb300/csrc/
mlp.cu): forward, loss, backward.

`quantized=True` mirrors the kernels' BF16 rounding points (weights, the
ReLU outputs H1/H2, dO, dZ2, dZ1) with all arithmetic in FP64, so the GPU
gradients differ from it only by FP32 accumulation; `quantized=False` is the
exact FP64 gradient of the same loss.
"""
from __future__ import annotations

import numpy as np

LAYOUT = [("W1", (128, 16)), ("b1", (128,)), ("W2", (128, 128)), ("b2", (128,)), ("W3", (32, 128)), ("b3", (32,))]


def unflatten(flat):
    out, o = {}, 0
    for name, shape in LAYOUT:
        size = int(np.prod(shape))
        out[name] = np.asarray(flat[o:o + size], dtype=np.float64).reshape(shape)
        o += size
    return out


def flatten(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in LAYOUT])


def bf16(x):
    """Round to bfloat16 (nearest, ties to even) and return as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


# ReLU hidden units, the function the engine's network uses
def relu(z):
    return np.maximum(z, 0.0)


def relu_grad(z):
    return (z > 0.0).astype(np.float64)


def softplus(x):
    return np.where(x > 20.0, x, np.log1p(np.exp(np.minimum(x, 20.0))))


def sigmoid(x):
    return 1.0 / (1.0 + np.exp(-x))


def forward(params, X, quantized=True):
    q = bf16 if quantized else (lambda a: np.asarray(a, dtype=np.float64))
    W1, W2, W3 = q(params["W1"]), q(params["W2"]), q(params["W3"])
    Z1 = X @ W1.T + params["b1"]
    H1 = q(relu(Z1))
    Z2 = H1 @ W2.T + params["b2"]
    H2 = q(relu(Z2))
    O = H2 @ W3.T + params["b3"]
    return {"Z1": Z1, "H1": H1, "Z2": Z2, "H2": H2, "O": O, "W1": W1, "W2": W2, "W3": W3}


def loss_and_grad(params, X, T, amp_weight=1.0, quantized=True):
    """Mean batch loss and the gradient of every parameter (dict)."""
    q = bf16 if quantized else (lambda a: np.asarray(a, dtype=np.float64))
    B = X.shape[0]
    f = forward(params, X, quantized)
    O = f["O"]
    z, y = O[:, :10], T[:, :10]
    o, t = O[:, 10:20], T[:, 10:20]
    sp = softplus(o)
    loss = (np.maximum(z, 0) - z * y + np.log1p(np.exp(-np.abs(z)))).sum() + amp_weight * ((sp - t) ** 2).sum()
    loss /= B
    dO = np.zeros_like(O)
    dO[:, :10] = (sigmoid(z) - y) / B
    dO[:, 10:20] = 2.0 * amp_weight * (sp - t) * sigmoid(o) / B
    dO = q(dO)
    g = {}
    g["W3"] = dO.T @ f["H2"]
    g["b3"] = dO.sum(axis=0)
    dH2 = dO @ f["W3"]
    dZ2 = q(dH2 * relu_grad(f["Z2"]))
    g["W2"] = dZ2.T @ f["H1"]
    g["b2"] = dZ2.sum(axis=0)
    dH1 = dZ2 @ f["W2"]
    dZ1 = q(dH1 * relu_grad(f["Z1"]))
    g["W1"] = dZ1.T @ X
    g["b1"] = dZ1.sum(axis=0)
    return loss, g


def loss_only(params, X, T, amp_weight=1.0):
    return loss_and_grad(params, X, T, amp_weight, quantized=False)[0]
