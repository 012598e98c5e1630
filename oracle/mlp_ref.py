"""FP64 numpy restatement of the learned-stop network (test infrastructure only): the checker
for the GPU forward / backward / Adam kernels (quantization_graph_gb300/csrc/mlp.cu).

Packed layout (weight matrices input-major): W1[8][64] b1[64] W2[64][64] b2[64] w3[64] b3,
W[in][out]. Inputs are standardised with
norm = (mean[8], inv_std[8]). Loss: mean binary cross-entropy with logits (the stop classifier)
or mean half squared error of the output (the hop budget).
"""
from __future__ import annotations

import numpy as np

IN, H = 8, 64
W1, B1 = 0, 64 * 8
W2 = B1 + 64
B2 = W2 + 64 * 64
W3 = B2 + 64
B3 = W3 + 64
PARAMS = B3 + 1


def unpack(w):
    w = np.asarray(w, np.float64)
    # returned as [out][in] matrices
    return (w[W1:B1].reshape(IN, H).T, w[B1:W2], w[W2:B2].reshape(H, H).T, w[B2:W3], w[W3:B3], w[B3])


def bf16_round(w32: np.ndarray) -> np.ndarray:
    """float32 -> bfloat16 (round to nearest even) -> float64."""
    b = np.ascontiguousarray(w32, np.float32).view(np.uint32).astype(np.uint64)
    rounded = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return rounded.astype(np.uint32).view(np.float32).astype(np.float64)


def forward(w, norm, x):
    a, b1, c, b2, d, b3 = unpack(w)
    f = (np.asarray(x, np.float64) - norm[:IN]) * norm[IN:]
    h1 = np.maximum(f @ a.T + b1, 0.0)
    h2 = np.maximum(h1 @ c.T + b2, 0.0)
    return h2 @ d + b3, (f, h1, h2)


def loss_and_grad(w, norm, x, y, mse=False):
    a, b1, c, b2, d, b3 = unpack(w)
    z, (f, h1, h2) = forward(w, norm, x)
    y = np.asarray(y, np.float64)
    n = len(y)
    if mse:
        loss = np.mean(0.5 * (z - y) ** 2)
        dz = (z - y) / n
    else:
        loss = np.mean(np.maximum(z, 0) - z * y + np.log1p(np.exp(-np.abs(z))))
        dz = (1.0 / (1.0 + np.exp(-z)) - y) / n
    g = np.zeros(PARAMS)
    g[B3] = dz.sum()
    g[W3:B3] = h2.T @ dz
    d2 = (dz[:, None] * d[None, :]) * (h2 > 0)
    g[B2:W3] = d2.sum(0)
    g[W2:B2] = (h1.T @ d2).ravel()
    d1 = (d2 @ c) * (h1 > 0)
    g[B1:W2] = d1.sum(0)
    g[W1:B1] = (f.T @ d1).ravel()
    return loss, g


def adam(master, grad, m, v, lr, beta1, beta2, eps, step):
    m = beta1 * m + (1 - beta1) * grad
    v = beta2 * v + (1 - beta2) * grad * grad
    upd = lr * (m / (1 - beta1 ** step)) / (np.sqrt(v / (1 - beta2 ** step)) + eps)
    return master - upd, m, v
