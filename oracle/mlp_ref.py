"""FP64 reference of the warm-start MLP (numpy), for checking the GPU kernels.

TEST INFRASTRUCTURE ONLY.  It mirrors the network of
tgvreconclaude_gb300/csrc/mlp.cu: inputs are BF16, the weights used by the
forward pass are the BF16-rounded parameters, hidden activations are rounded to
BF16 after the ReLU, accumulation is exact here (FP64) and FP32 on the GPU.
Gradients treat the BF16 rounding as the identity, as the GPU backward pass does.
"""
from __future__ import annotations

import numpy as np

K1, H = 16, 64
P_W1 = 0
P_B1 = P_W1 + K1 * H
P_W2 = P_B1 + H
P_B2 = P_W2 + H * H
P_W3 = P_B2 + H
P_B3 = P_W3 + H
P_N = P_B3 + 1


def bf16_round(x):
    """float32 -> nearest-even bfloat16 value, returned as float32."""
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def bf16_bits_to_float(xb):
    """uint16 bf16 bit patterns -> float32 values."""
    return (np.asarray(xb, np.uint32) << 16).view(np.float32)


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[P_W1:P_B1].reshape(K1, H), p[P_B1:P_W2], p[P_W2:P_B2].reshape(H, H), p[P_B2:P_W3],
            p[P_W3:P_B3], p[P_B3])


def forward(p, X, rnd=True):
    """X: (n, 16) float (already bf16 values).  Returns y and the activations.
    rnd=False drops the BF16 rounding (a plain FP64 network)."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    R = (lambda a: bf16_round(a.astype(np.float32)).astype(np.float64)) if rnd else (lambda a: a)
    W1r, W2r, W3r = R(W1), R(W2), R(W3)
    X = np.asarray(X, np.float64)
    z1 = X @ W1r + b1
    h1 = R(np.maximum(z1, 0))
    z2 = h1 @ W2r + b2
    h2 = R(np.maximum(z2, 0))
    y = h2 @ W3r + b3
    return y, (X, h1, h2, W2r, W3r)


def loss_and_grad(p, X, t, rnd=True):
    y, (Xd, h1, h2, W2r, W3r) = forward(p, X, rnd)
    m = len(t)
    e = y - np.asarray(t, np.float64)
    dy = 2.0 * e / m
    g = np.zeros(P_N)
    g[P_W3:P_B3] = h2.T @ dy
    g[P_B3] = dy.sum()
    dz2 = np.outer(dy, W3r) * (h2 > 0)
    g[P_W2:P_B2] = (h1.T @ dz2).ravel()
    g[P_B2:P_W3] = dz2.sum(0)
    dz1 = (dz2 @ W2r.T) * (h1 > 0)
    g[P_W1:P_B1] = (Xd.T @ dz1).ravel()
    g[P_B1:P_W2] = dz1.sum(0)
    return float((e * e).mean()), g
