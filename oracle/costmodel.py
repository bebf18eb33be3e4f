"""CPU FP64 oracle of the autotuner's cost model (test infrastructure only:
tests use it to check the device kernels; the library never calls it).

The reference has no learned component, so there is no reference file to
follow: this module states the network's definition -- n_in -> 64 -> 64 -> 1,
tanh hidden units, mean-squared-error loss over the data set, Adam with
beta1 0.9, beta2 0.999, eps 1e-8 -- in plain numpy, and its analytic
gradient is pinned to the definition of a derivative by central finite
differences (fd_grad), which the CPU tests check.

Parameter vector layout (flat): W1 [n_in][64], b1 [64], W2 [64][64],
b2 [64], w3 [64], b3.
"""
import numpy as np

H = 64


def n_params(d):
    return d * H + H + H * H + H + H + 1


def unpack(p, d):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + d * H].reshape(d, H); o += d * H
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def pack(W1, b1, W2, b2, w3, b3):
    return np.concatenate([W1.ravel(), b1, W2.ravel(), b2, w3, [b3]])


def forward(p, X):
    X = np.asarray(X, dtype=np.float64)
    W1, b1, W2, b2, w3, b3 = unpack(p, X.shape[1])
    h1 = np.tanh(X @ W1 + b1)
    h2 = np.tanh(h1 @ W2 + b2)
    return h2 @ w3 + b3


def loss(p, X, t):
    e = forward(p, X) - np.asarray(t, dtype=np.float64)
    return float(np.mean(e * e))


def loss_grad(p, X, t):
    """(loss, gradient) by backpropagation, FP64."""
    X = np.asarray(X, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    n = X.shape[0]
    W1, b1, W2, b2, w3, b3 = unpack(p, X.shape[1])
    h1 = np.tanh(X @ W1 + b1)
    h2 = np.tanh(h1 @ W2 + b2)
    e = h2 @ w3 + b3 - t
    dy = 2.0 * e / n
    g2 = dy[:, None] * w3[None, :] * (1.0 - h2 * h2)
    g1 = (g2 @ W2.T) * (1.0 - h1 * h1)
    grad = pack(X.T @ g1, g1.sum(0), h1.T @ g2, g2.sum(0), h2.T @ dy, dy.sum())
    return float(np.mean(e * e)), grad


def fd_grad(p, X, t, eps=1e-6, idx=None):
    """Central finite differences of the loss at the parameters in idx (all
    when None)."""
    p = np.asarray(p, dtype=np.float64).copy()
    idx = range(p.size) if idx is None else idx
    out = {}
    for i in idx:
        v = p[i]
        p[i] = v + eps
        lp = loss(p, X, t)
        p[i] = v - eps
        lm = loss(p, X, t)
        p[i] = v
        out[i] = (lp - lm) / (2 * eps)
    return out


def adam_train(p, X, t, steps, lr):
    """Full-batch Adam from a fresh optimiser state; returns (params, losses
    before each step)."""
    p = np.asarray(p, dtype=np.float64).copy()
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    b1, b2, eps = 0.9, 0.999, 1e-8
    losses = []
    for k in range(1, steps + 1):
        l, g = loss_grad(p, X, t)
        losses.append(l)
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        p -= lr * (m / (1 - b1 ** k)) / (np.sqrt(v / (1 - b2 ** k)) + eps)
    return p, losses
