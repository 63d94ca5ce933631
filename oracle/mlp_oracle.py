"""CPU oracle for the learned-guess network -- TEST INFRASTRUCTURE ONLY.

FP64 NumPy forward and backward of the pair MLP (dense layers, SiLU between them,
masked mean squared error), used to check the GPU kernels' outputs and gradients.
Weights are taken as given (the caller passes the BF16-rounded weights the kernels
multiply with)."""
import numpy as np


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(X, Ws, bs):
    A = X.astype(np.float64)
    cache = []
    for k, (W, b) in enumerate(zip(Ws, bs)):
        Z = A @ W + b
        cache.append((A, Z))
        A = silu(Z) if k < len(Ws) - 1 else Z
    return A, cache


def loss_and_grads(X, T, mask, Ws, bs):
    Y, cache = forward(X, Ws, bs)
    cnt = max(mask.sum(), 1.0)
    d = (Y - T) * mask
    loss = (d * d).sum() / cnt
    G = 2.0 * d / cnt
    grads = [None] * len(Ws)
    for k in reversed(range(len(Ws))):
        A, Z = cache[k]
        if k < len(Ws) - 1:
            G = G * dsilu(Z)
        grads[k] = (A.T @ G, G.sum(axis=0))
        G = G @ Ws[k].T
    return loss, Y, grads
