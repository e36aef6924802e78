"""CPU oracle of the learned-guess network (TEST INFRASTRUCTURE ONLY).

A float64 numpy restatement of the 3-layer MLP of the GPU guess (SiLU hidden
layers, identity output, masked mean-squared error) with its analytic backward
pass.  The GPU forward/backward kernels (csrc/mlp.cu, driven by mmd/guess.py) are
checked against it on the same BF16-rounded weights.
"""
import numpy as np


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(W, b, X):
    acts = []
    h = X
    for i in range(3):
        z = h @ W[i].T + b[i]
        y = silu(z) if i < 2 else z
        acts.append((h, z, y))
        h = y
    return acts


def loss_and_grads(W, b, X, T, M):
    acts = forward(W, b, X)
    Y = acts[-1][2]
    cnt = max(M.sum(), 1.0)
    d = (Y - T) * M
    loss = float((d * d).sum() / cnt)
    dY = 2.0 * d / cnt
    grads = [None] * 3
    g = dY
    for i in (2, 1, 0):
        h, z, _ = acts[i]
        dz = g * dsilu(z) if i < 2 else g
        grads[i] = (dz.T @ h, dz.sum(axis=0))
        g = dz @ W[i]
    return loss, grads
