"""TEST INFRASTRUCTURE: FP64 numpy restatement of the learned predictor's dense network.

Same architecture and parameter layout as the device network (per layer W (out x in, row-major) then b (out);
GELU (erf form) after every hidden layer; linear output; mean-squared-error loss over all outputs).  The
device forward pass multiplies with the BF16 rounding of the FP32 master weights and back-propagates through
them unchanged (straight-through), so the oracle rounds the weights the same way.  Used only to check the
device forward pass and gradients.
"""
from __future__ import annotations

import math

import numpy as np


def bf16_round(x):
    """Round-to-nearest-even of FP32 values to BF16, returned as FP32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return r.astype(np.uint32).view(np.float32)


def layer_dims(n_in, width, depth, n_out):
    return [n_in] + [width] * depth + [n_out]


def unpack(params, dims):
    out, o = [], 0
    for a, b in zip(dims[:-1], dims[1:]):
        W = params[o:o + a * b].reshape(b, a)
        o += a * b
        bias = params[o:o + b]
        o += b
        out.append((W, bias))
    return out


_erf = np.vectorize(math.erf)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def forward(params, dims, x):
    layers = unpack(np.asarray(params, dtype=np.float32), dims)
    h = np.asarray(x, dtype=np.float64)
    for i, (W, b) in enumerate(layers):
        z = h @ bf16_round(W).astype(np.float64).T + b.astype(np.float64)
        h = gelu(z) if i + 1 < len(layers) else z
    return h


def loss_grad(params, dims, x, t):
    layers = unpack(np.asarray(params, dtype=np.float32), dims)
    Ws = [bf16_round(W).astype(np.float64) for W, _ in layers]
    bs = [b.astype(np.float64) for _, b in layers]
    h = [np.asarray(x, dtype=np.float64)]
    zs = []
    for i in range(len(layers)):
        z = h[-1] @ Ws[i].T + bs[i]
        zs.append(z)
        h.append(gelu(z) if i + 1 < len(layers) else z)
    y = h[-1]
    t = np.asarray(t, dtype=np.float64)
    n = y.size
    loss = float(((y - t) ** 2).sum() / n)
    dy = 2.0 * (y - t) / n
    grads = []
    for i in reversed(range(len(layers))):
        dz = dy if i + 1 == len(layers) else dy * gelu_grad(zs[i])
        grads.append((dz.T @ h[i], dz.sum(axis=0)))
        dy = dz @ Ws[i]
    grads.reverse()
    return loss, np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
