"""FP64 restatement of the transport surrogate's network (TEST INFRASTRUCTURE ONLY: the checker of the
GPU forward and backward kernels; the product library never uses it).

The surrogate has no reference counterpart. Network: layers l = 0 .. L-1, Z_l = A_l W_l^T + b_l,
A_{l+1} = silu(Z_l) for hidden layers, the last layer linear; loss = mean over rows and valid output
columns of (y - t)^2. With ``bf16=True`` the values the GPU stores in BF16 are rounded the same way
(features, weights, hidden activations, the SiLU derivatives at the pre-activations, the loss gradient
and the back-propagated pre-activation gradients, round-to-nearest-even), so that the remaining
difference is FP32 accumulation (and the GPU's approximate tanh) only.
"""
from __future__ import annotations

import numpy as np


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((a + 0x7FFF + ((a >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(layers, X, bf=False):
    """Network outputs [rows, n_out] for features X [rows, n_in]; layers = [(W [out, in], b [out])]."""
    r = bf16 if bf else (lambda v: np.asarray(v, dtype=np.float64))
    A = r(X)
    for l, (W, b) in enumerate(layers):
        Z = A @ r(W).T + np.asarray(b, dtype=np.float64)
        if l == len(layers) - 1:
            return Z
        A = r(silu(Z))


def loss_and_grads(layers, X, T, n_valid, bf=False):
    """(loss, [(dW, db)] per layer, outputs) of the mean squared error over the first n_valid columns."""
    r = bf16 if bf else (lambda v: np.asarray(v, dtype=np.float64))
    rows = X.shape[0]
    As, Zs = [r(X)], []
    for l, (W, b) in enumerate(layers):
        Z = As[-1] @ r(W).T + np.asarray(b, dtype=np.float64)
        if l == len(layers) - 1:
            Y = Z
            break
        Zs.append(Z)
        As.append(r(silu(Z)))
    D = np.zeros_like(Y)
    D[:, :n_valid] = Y[:, :n_valid] - np.asarray(T, dtype=np.float64)[:, :n_valid]
    loss = float((D[:, :n_valid] ** 2).sum() / (rows * n_valid))
    G = r(D * (2.0 / (rows * n_valid)))
    grads = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        grads[l] = (G.T @ As[l], G.sum(axis=0))
        if l == 0:
            break
        dA = G @ r(layers[l][0])
        G = r(dA * r(dsilu(Zs[l - 1])))
    return loss, grads, Y
