"""CPU oracle of the warm-start network (float64 numpy), for checking the GPU
kernels in suqa_gb300/csrc/sq_mlp.cu.  TEST INFRASTRUCTURE ONLY.

Same function and rounding points as the kernels: the input, the weights, the
biases and every hidden activation are rounded to BF16 (round to nearest even);
pre-activations and all sums are kept in float64 here (FP32 on the GPU).
gelu(z) = z * Phi(z).  Loss = mean over rows of sum_k mask * (y - t)^2.
"""
from __future__ import annotations

import math

import numpy as np


def bf16(x):
    x = np.asarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (u & 0xFFFFFFFF).astype(np.uint32).view(np.float32).astype(np.float64)


_erf = np.vectorize(math.erf)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    cdf = 0.5 * (1.0 + _erf(z / math.sqrt(2.0)))
    pdf = np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)
    return cdf + z * pdf


def unpack(flat, dims):
    out, off = [], 0
    for l in range(len(dims) - 1):
        n_w = dims[l] * dims[l + 1]
        W = flat[off:off + n_w].reshape(dims[l + 1], dims[l])
        off += n_w
        b = flat[off:off + dims[l + 1]]
        off += dims[l + 1]
        out.append((W, b))
    return out


def forward_backward(flat, dims, x, t, mask=None):
    """Returns (y, loss, flat gradient)."""
    layers = unpack(np.asarray(flat, dtype=np.float64), dims)
    a = bf16(x)
    acts, zs = [a], []
    for l, (W, b) in enumerate(layers):
        z = a @ bf16(W).T + bf16(b)
        zs.append(z)
        if l + 1 < len(layers):
            a = bf16(gelu(z))
            acts.append(a)
        else:
            y = z
    B = x.shape[0]
    m = np.ones_like(y) if mask is None else mask
    loss = float(np.sum(m * (y - t) ** 2) / B)
    d = 2.0 * m * (y - t) / B
    grads = []
    for l in range(len(layers) - 1, -1, -1):
        W, b = layers[l]
        gW = d.T @ acts[l]
        gb = d.sum(axis=0)
        grads.append((gW, gb))
        if l > 0:
            d = (d @ bf16(W)) * gelu_grad(zs[l - 1])
    grads.reverse()
    flat_g = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return y, loss, flat_g
