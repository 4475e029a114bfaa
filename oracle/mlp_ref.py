"""Float64 numpy restatement of the learned-guess network (tests only).

Same architecture and conventions as gpu4pyscf_gb300/scf/mlp.py: dense
layers y = x W + b, SiLU (x * sigmoid(x)) between layers, linear output;
masked mean-squared error mean(mask * (y - t)^2) over the mask's support.
Used to check the GPU kernels' forward pass and gradients; the gradients
here are pinned against central finite differences in
tests/test_mlp.py.
"""
import numpy as np


def silu(z):
    return z / (1. + np.exp(-z))


def dsilu(z):
    s = 1. / (1. + np.exp(-z))
    return s + z * s * (1. - s)


def forward(W, b, X):
    h = np.asarray(X, dtype=np.float64)
    xs, zs = [h], []
    for l in range(len(W)):
        z = h @ W[l] + b[l]
        if l == len(W) - 1:
            return z, (xs, zs)
        zs.append(z)
        h = silu(z)
        xs.append(h)


def loss(W, b, X, T, mask=None):
    y, _ = forward(W, b, X)
    m = np.ones_like(y) if mask is None else mask
    return float(np.sum(m * (y - T) ** 2) / np.sum(m))


def grads(W, b, X, T, mask=None):
    y, (xs, zs) = forward(W, b, X)
    m = np.ones_like(y) if mask is None else mask
    g = 2. * m * (y - T) / np.sum(m)
    gW, gb = [None] * len(W), [None] * len(W)
    for l in reversed(range(len(W))):
        if l < len(W) - 1:
            g = g * dsilu(zs[l])
        gW[l] = xs[l].T @ g
        gb[l] = g.sum(0)
        g = g @ W[l].T
    return gW, gb, g
