"""CPU oracle of the warm-start network (reprobus_gb300/csrc/mlp_kernels.cu).

TEST INFRASTRUCTURE ONLY: the tests use it to check the GPU forward pass and
the gradients of the GPU training kernels; the product never calls it.

It restates the network in float64 numpy and rounds to BF16 exactly where
the GPU kernels store BF16 (normalised inputs, weights, hidden activations,
the gradients of the pre-activations), so that the remaining difference is
FP32 accumulation on the tensor cores against float64 here.
"""
from __future__ import annotations

import numpy as np

DIMS = [(64, 256), (256, 256), (256, 256), (256, 64)]
NY = 57


def bf16(a):
    """Round to bfloat16 (round to nearest even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    out, o = [], 0
    for i, n in DIMS:
        W = np.asarray(params[o:o + i * n], dtype=np.float64).reshape(n, i)
        o += i * n
        out.append((W, np.asarray(params[o:o + n], dtype=np.float64)))
        o += n
    return out


def _silu(z):
    return z / (1.0 + np.exp(-z))


def _dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(params, norm, X, keep=False):
    """Raw outputs (B x 64) for raw features X; keep: also the per-layer
    (input, pre-activation) pairs."""
    layers = unpack(params)
    xm, xs, ym, ys = norm[:64], norm[64:128], norm[128:192], norm[192:256]
    xn = (np.asarray(X, np.float32) - xm.astype(np.float32)) / xs.astype(np.float32)
    hi = bf16(xn)
    lo = bf16(xn.astype(np.float64) - hi)
    A = hi + lo  # layer 0 sees the BF16 pair hi + lo of each normalised feature
    saved = []
    for l, (W, b) in enumerate(layers):
        Z = A @ bf16(W).T + b
        saved.append((A, Z))
        A = bf16(_silu(Z)) if l < len(layers) - 1 else Z
    out = A * ys + ym
    if len(norm) > 256:
        out = np.where(np.abs(out) >= norm[256:320], out, 0.0)
    out[:, NY:] = 0.0
    return (out, saved) if keep else out


def loss_and_grads(params, norm, X, Y):
    """Mean squared error of the normalised outputs over the 57 used columns,
    and its gradient packed like the parameters."""
    layers = unpack(params)
    _, saved = forward(params, norm, X, keep=True)
    ym, ys = norm[128:192], norm[192:256]
    B = X.shape[0]
    yn = (np.asarray(Y, np.float32) - ym.astype(np.float32)) / ys.astype(np.float32)
    Z3 = saved[-1][1]
    d = np.zeros_like(Z3)
    d[:, :NY] = Z3[:, :NY] - yn[:, :NY]
    loss = float((d ** 2).sum() / (B * NY))
    dZ = bf16(2.0 * d / (B * NY))
    grads = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        A, _ = saved[l]
        W, _ = layers[l]
        grads[l] = (dZ.T @ A, dZ.sum(0))
        if l > 0:
            dZ = bf16((dZ @ bf16(W)) * _dsilu(saved[l - 1][1]))
    packed = np.concatenate([np.concatenate([g[0].ravel(), g[1]]) for g in grads])
    return loss, packed
