"""ORACLE -- test infrastructure, not product code.

FP64 numpy forward and backward of the tail-surrogate MLP (GELU hidden
layers, linear output, weighted MSE loss), the yardstick for the gradient
checks of tfce_mediation_gb300/csrc/mlp.cu."""
import math

import numpy as np

_erf = np.vectorize(math.erf)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    cdf = 0.5 * (1.0 + _erf(x / math.sqrt(2.0)))
    pdf = np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)
    return cdf + x * pdf


def forward(Ws, bs, X):
    h = np.asarray(X, np.float64)
    tape = []
    for i, (W, b) in enumerate(zip(Ws, bs)):
        z = h @ W + b
        tape.append((h, z))
        h = z if i == len(Ws) - 1 else gelu(z)
    return h, tape


def loss_and_grads(Ws, bs, X, T, col_weight=None):
    Ws = [np.asarray(W, np.float64) for W in Ws]
    bs = [np.asarray(b, np.float64) for b in bs]
    y, tape = forward(Ws, bs, X)
    w = np.ones(y.shape[1]) if col_weight is None else np.asarray(col_weight, np.float64)
    d = y - T
    n = y.size
    loss = float(np.sum(d * d * w) / n)
    dy = 2.0 * d * w / n
    gW, gb = [None] * len(Ws), [None] * len(Ws)
    for i in reversed(range(len(Ws))):
        h, z = tape[i]
        dz = dy if i == len(Ws) - 1 else dy * gelu_grad(z)
        gW[i] = h.T @ dz
        gb[i] = dz.sum(axis=0)
        dy = dz @ Ws[i].T
    return loss, gW, gb, y
