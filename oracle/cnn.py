"""ORACLE for the learned estimator's network — test infrastructure only.

A float64 NumPy restatement of the CNN of oct_recon_af_v1_gb300/learned.py
(conv 3x3 pad 1 -> ReLU -> 2x2 mean pool, x4; dense -> ReLU -> dense; MSE),
forward and backward, for the gradient checks of the CUDA kernels.  The
reference has no learned estimator, so nothing here restates reference code;
the gradients are checked against finite differences of this forward pass.
"""
from __future__ import annotations

import numpy as np


def conv3x3(x, w, b):
    """x (n, C, H, W), w (K, C, 3, 3), b (K) -> (n, K, H, W), zero padding 1."""
    n, C, H, W = x.shape
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1)))
    y = np.zeros((n, w.shape[0], H, W))
    for i in range(3):
        for j in range(3):
            y += np.einsum("nchw,kc->nkhw", xp[:, :, i:i + H, j:j + W], w[:, :, i, j])
    return y + b[None, :, None, None]


def conv3x3_bwd(x, w, dy):
    n, C, H, W = x.shape
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1)))
    dw = np.zeros_like(w)
    dxp = np.zeros_like(xp)
    for i in range(3):
        for j in range(3):
            dw[:, :, i, j] = np.einsum("nkhw,nchw->kc", dy, xp[:, :, i:i + H, j:j + W])
            dxp[:, :, i:i + H, j:j + W] += np.einsum("nkhw,kc->nchw", dy, w[:, :, i, j])
    return dxp[:, :, 1:-1, 1:-1], dw, dy.sum(axis=(0, 2, 3))


def relu_pool(y):
    r = np.maximum(y, 0.0)
    n, K, H, W = r.shape
    return r.reshape(n, K, H // 2, 2, W // 2, 2).mean(axis=(3, 5))


def relu_pool_bwd(dp, y):
    g = np.repeat(np.repeat(dp, 2, axis=2), 2, axis=3) * 0.25
    return np.where(y > 0, g, 0.0)


def forward(params, x):
    """params: [w0, b0, ..., w3, b3, W1, b1, W2, b2]; returns (pred, cache)."""
    cache = {"x": x, "pre": [], "pooled": []}
    cur = x
    for i in range(4):
        y = conv3x3(cur, params[2 * i], params[2 * i + 1])
        cur = relu_pool(y)
        cache["pre"].append(y)
        cache["pooled"].append(cur)
    flat = cur.reshape(cur.shape[0], -1)
    h_pre = flat @ params[8].T + params[9]
    h = np.maximum(h_pre, 0.0)
    out = h @ params[10].T + params[11]
    cache.update(flat=flat, h_pre=h_pre, h=h)
    return out, cache


def mse(pred, target):
    d = pred - target
    return float(np.mean(d * d)), 2.0 * d / d.size


def backward(params, cache, dout):
    grads = [None] * len(params)
    grads[10] = dout.T @ cache["h"]
    grads[11] = dout.sum(0)
    dh = (dout @ params[10]) * (cache["h_pre"] > 0)
    grads[8] = dh.T @ cache["flat"]
    grads[9] = dh.sum(0)
    dp = (dh @ params[8]).reshape(cache["pooled"][-1].shape)
    for i in reversed(range(4)):
        dy = relu_pool_bwd(dp, cache["pre"][i])
        xin = cache["x"] if i == 0 else cache["pooled"][i - 1]
        dx, grads[2 * i], grads[2 * i + 1] = conv3x3_bwd(xin, params[2 * i], dy)
        dp = dx
    return grads
