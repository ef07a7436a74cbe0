"""FP64 NumPy restatement of the transmit-field surrogate network (test infrastructure only):
random Fourier features -> 4 x (Linear 256 + SiLU) -> Linear 2, mean-squared loss
sum((out - y)^2) / (2 n).  Used to check the gradients of the GPU forward/backward kernels."""

import numpy as np


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def features(u, bmat):
    t = u @ bmat.T
    return np.concatenate([np.sin(2 * np.pi * t), np.cos(2 * np.pi * t)], axis=1)


def forward(u, bmat, W, b):
    a = features(u, bmat)
    acts, zs = [a], []
    for w, bb in zip(W[:-1], b[:-1]):
        z = a @ w.T + bb
        a = silu(z)
        zs.append(z)
        acts.append(a)
    out = a @ W[-1].T + b[-1]
    return out, acts, zs


def loss_and_grads(u, y, bmat, W, b):
    out, acts, zs = forward(u, bmat, W, b)
    n = u.shape[0]
    diff = out - y
    loss = float(np.sum(diff * diff)) / (2 * n)
    d = diff / n
    gW = [None] * len(W)
    gb = [None] * len(W)
    gW[-1] = d.T @ acts[-1]
    gb[-1] = d.sum(0)
    da = d @ W[-1]
    for layer in range(len(W) - 2, -1, -1):
        dz = da * silu_grad(zs[layer])
        gW[layer] = dz.T @ acts[layer]
        gb[layer] = dz.sum(0)
        da = dz @ W[layer]
    return loss, gW, gb
