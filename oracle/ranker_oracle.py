"""ORACLE — test infrastructure only: a float64 numpy restatement of the
candidate ranker's MLP (forward pass, weighted logistic loss and backward
pass), the CPU checker of the library's GPU training kernels. The reference
has no learned component; this oracle follows the model as the library
defines it:

    x[16] -> h = relu(W1 x + b1), W1[64][16] -> z = w2 . h + b2
    loss = mean_i w_i * (softplus(z_i) - y_i z_i)

with the weights W1 and w2 rounded to bf16 (round to nearest even) in the
forward pass and the gradient taken with respect to the fp32 master
parameters (straight through the rounding). Parameter layout:
W1 (row-major, 1024) | b1 (64) | w2 (64) | b2 (1).
"""

from __future__ import annotations

import numpy as np

FEAT = 16
HIDDEN = 64
W1, B1, W2, B2 = 0, HIDDEN * FEAT, HIDDEN * FEAT + HIDDEN, HIDDEN * FEAT + 2 * HIDDEN
PARAMS = B2 + 1


def bf16_round(a: np.ndarray) -> np.ndarray:
    """float32 -> bf16 -> float32, round to nearest even (finite inputs)."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) & 0xFFFF0000).astype(np.uint32).view(np.float32)


def unpack(params: np.ndarray, round_bf16: bool = True):
    p = np.asarray(params, np.float32)
    w1 = p[W1:B1]
    w2 = p[W2:B2]
    if round_bf16:
        w1, w2 = bf16_round(w1), bf16_round(w2)
    return (w1.astype(np.float64).reshape(HIDDEN, FEAT), p[B1:W2].astype(np.float64), w2.astype(np.float64),
            float(p[B2]))


def forward(params, x, round_bf16: bool = True) -> np.ndarray:
    w1, b1, w2, b2 = unpack(params, round_bf16)
    a = np.asarray(x, np.float64) @ w1.T + b1
    return np.maximum(a, 0.0) @ w2 + b2


def loss_and_grad(params, x, y, w=None, round_bf16: bool = True) -> tuple[float, np.ndarray, np.ndarray]:
    """Mean weighted logistic loss, its gradient w.r.t. the master params,
    and the logits."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    n = len(y)
    wt = np.ones(n) if w is None else np.asarray(w, np.float64)
    w1, b1, w2, b2 = unpack(params, round_bf16)
    a = x @ w1.T + b1
    h = np.maximum(a, 0.0)
    z = h @ w2 + b2
    softplus = np.maximum(z, 0.0) + np.log1p(np.exp(-np.abs(z)))
    loss = float(np.sum(wt * (softplus - y * z)) / n)
    dz = wt * (1.0 / (1.0 + np.exp(-z)) - y) / n
    dh = np.where(a > 0.0, dz[:, None] * w2[None, :], 0.0)
    g = np.zeros(PARAMS)
    g[W1:B1] = (dh.T @ x).reshape(-1)
    g[B1:W2] = dh.sum(axis=0)
    g[W2:B2] = (dz[:, None] * h).sum(axis=0)
    g[B2] = dz.sum()
    return loss, g, z


def init_params(seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    p = np.zeros(PARAMS, np.float32)
    a1 = np.sqrt(6.0 / (FEAT + HIDDEN))
    p[W1:B1] = rng.uniform(-a1, a1, HIDDEN * FEAT)
    p[B1:W2] = rng.uniform(-0.1, 0.1, HIDDEN)
    a2 = np.sqrt(6.0 / (HIDDEN + 1))
    p[W2:B2] = rng.uniform(-a2, a2, HIDDEN)
    p[B2] = 0.05
    return p
