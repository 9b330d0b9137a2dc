"""FP64 numpy restatement of the neighbour-radius MLP (TEST INFRASTRUCTURE
ONLY): forward pass and the gradient of mean w (y - t)^2, for checking the
GPU training kernels (csrc/rsmlp.cu).  The weight matrices are taken as the
kernels see them (BF16-rounded values), the biases as FP32."""
from __future__ import annotations

import math

import numpy as np

H, I = 64, 8


def unpack(w):
    o = 0
    W1 = w[o:o + H * I].reshape(H, I); o += H * I
    b1 = w[o:o + H]; o += H
    W2 = w[o:o + H * H].reshape(H, H); o += H * H
    b2 = w[o:o + H]; o += H
    W3 = w[o:o + H]; o += H
    b3 = w[o]
    return W1, b1, W2, b2, W3, b3


# GELU in its tanh form (Hendrycks and Gimpel, 2016), as the kernels define it
_C = math.sqrt(2.0 / math.pi)
_A = 0.044715


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(_C * (x + _A * x ** 3)))


def gelu_grad(x):
    t = np.tanh(_C * (x + _A * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * _C * (1.0 + 3.0 * _A * x * x)


def forward(wq, wf, X):
    W1, _, W2, _, W3, _ = unpack(np.asarray(wq, dtype=np.float64))
    _, b1, _, b2, _, b3 = unpack(np.asarray(wf, dtype=np.float64))
    X = np.asarray(X, dtype=np.float64)
    z1 = X @ W1.T + b1
    h1 = gelu(z1)
    z2 = h1 @ W2.T + b2
    h2 = gelu(z2)
    return h2 @ W3 + b3, (z1, h1, z2, h2)


def gradient(wq, wf, X, T, W=None):
    """Returns (grad [P] in the kernel's parameter order, loss)."""
    Wm1, _, Wm2, _, Wm3, _ = unpack(np.asarray(wq, dtype=np.float64))
    X = np.asarray(X, dtype=np.float64)
    B = X.shape[0]
    w = np.ones(B) if W is None else np.asarray(W, dtype=np.float64)
    y, (z1, h1, z2, h2) = forward(wq, wf, X)
    r = y - np.asarray(T, dtype=np.float64)
    loss = float(np.sum(w * r * r) / B)
    dy = 2.0 * w * r / B
    dW3 = h2.T @ dy
    db3 = dy.sum()
    dz2 = (dy[:, None] * Wm3[None, :]) * gelu_grad(z2)
    dW2 = dz2.T @ h1
    db2 = dz2.sum(0)
    dz1 = (dz2 @ Wm2) * gelu_grad(z1)
    dW1 = dz1.T @ X
    db1 = dz1.sum(0)
    g = np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dW3, [db3]])
    return g, loss
