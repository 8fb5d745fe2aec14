"""CPU restatement of the learned stage guess's network (numpy).

TEST INFRASTRUCTURE ONLY: the checker for the library's BF16 tensor-core
MLP (``sem_learner_*``).  The reference has no learned component, so this
oracle follows the library's own definition (include/sem_gb300.h, learned
stage guess): a ReLU MLP d_in -> H -> H -> d_out, weights [in][out], trained
on the mean-squared error with Adam.  Like the CUDA path it rounds every
GEMM operand to BF16 (round to nearest even) and accumulates in higher
precision; the ReLU masks, bias gradients and Adam update use FP32 values.

Parity is pinned two ways: ``grads_fp64`` (no BF16 rounding) is checked
against central finite differences of ``loss_fp64`` on the CPU, and the BF16
forward/backward is the same algebra with the rounding inserted.
"""
from __future__ import annotations

import numpy as np


def bf16_round(a) -> np.ndarray:
    """float32 values rounded to the nearest BF16 (ties to even), as float32"""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) & 0xFFFF0000).astype(np.uint32)
    out = r.view(np.float32).copy()
    nan = np.isnan(a)
    out[nan] = a[nan]
    return out


def _mm(a, b, bf16: bool):
    if bf16:
        a, b = bf16_round(a), bf16_round(b)
    return (a.astype(np.float64) @ b.astype(np.float64)).astype(np.float32)


def forward(x, params, bf16: bool = True):
    """params = [(W1, b1), (W2, b2), (W3, b3)]; returns (out, cache)"""
    (W1, b1), (W2, b2), (W3, b3) = params
    h1 = np.maximum(_mm(x, W1, bf16) + b1, 0.0).astype(np.float32)
    h2 = np.maximum(_mm(h1, W2, bf16) + b2, 0.0).astype(np.float32)
    out = (_mm(h2, W3, bf16) + b3).astype(np.float32)
    return out, (x, h1, h2)


def loss_and_grads(x, target, params, bf16: bool = True):
    """mean((out - target)^2) and [(gW, gb)] per layer"""
    (W1, _), (W2, _), (W3, _) = params
    out, (x, h1, h2) = forward(x, params, bf16)
    n = out.size
    e = (out - target).astype(np.float32)
    loss = float(np.sum(e.astype(np.float64) ** 2) / n)
    d = (np.float32(2.0 / n) * e).astype(np.float32)
    gW3 = _mm(h2.T, d, bf16)
    gb3 = d.sum(axis=0, dtype=np.float64).astype(np.float32)
    d2 = _mm(d, W3.T, bf16) * (h2 > 0)
    gW2 = _mm(h1.T, d2, bf16)
    gb2 = d2.sum(axis=0, dtype=np.float64).astype(np.float32)
    d1 = _mm(d2, W2.T, bf16) * (h1 > 0)
    gW1 = _mm(x.T, d1, bf16)
    gb1 = d1.sum(axis=0, dtype=np.float64).astype(np.float32)
    return loss, [(gW1, gb1), (gW2, gb2), (gW3, gb3)]


def loss_fp64(x, target, params) -> float:
    h = x.astype(np.float64)
    for l, (W, b) in enumerate(params):
        h = h @ W.astype(np.float64) + b.astype(np.float64)
        if l < 2:
            h = np.maximum(h, 0.0)
    return float(np.mean((h - target) ** 2))


def grads_fp64(x, target, params):
    """exact backpropagation in float64 (for the finite-difference pin)"""
    hs = [x.astype(np.float64)]
    h = hs[0]
    for l, (W, b) in enumerate(params):
        h = h @ W.astype(np.float64) + b.astype(np.float64)
        if l < 2:
            h = np.maximum(h, 0.0)
        hs.append(h)
    d = 2.0 * (hs[-1] - target) / hs[-1].size
    grads = [None] * 3
    for l in (2, 1, 0):
        W = params[l][0].astype(np.float64)
        grads[l] = (hs[l].T @ d, d.sum(axis=0))
        if l > 0:
            d = (d @ W.T) * (hs[l] > 0)
    return grads


def adam_update(w, g, m, v, t: int, lr: float, b1=0.9, b2=0.999, eps=1e-8):
    """one Adam step in FP32 (bias-corrected moments); returns (w, m, v)"""
    f = np.float32
    m = (f(b1) * m + f(1 - b1) * g).astype(np.float32)
    v = (f(b2) * v + f(1 - b2) * g * g).astype(np.float32)
    c1 = f(1 - b1 ** t)
    c2 = f(1 - b2 ** t)
    w = (w - f(lr) * (m / c1) / (np.sqrt(v / c2) + f(eps))).astype(np.float32)
    return w, m, v
