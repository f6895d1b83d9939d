"""TEST INFRASTRUCTURE ONLY -- numpy float64 restatement of the learned planner's MLP
(3 layers, ReLU, mean squared error), the oracle for the gradient check of the CUDA
training kernels (erdos-selfridge_gb300/csrc/es_mlp.cu).  No reference counterpart: the
reference planner has no learned part.  Parameter layout: W1[H][D], b1[H], W2[H][H], b2[H],
W3[O][H], b3[O], flat."""
from __future__ import annotations

import numpy as np


def unpack(P, D, H, O):
    P = np.asarray(P, dtype=np.float64)
    i = 0

    def take(n, shape):
        nonlocal i
        a = P[i:i + n].reshape(shape)
        i += n
        return a
    W1 = take(H * D, (H, D)); b1 = take(H, (H,))
    W2 = take(H * H, (H, H)); b2 = take(H, (H,))
    W3 = take(O * H, (O, H)); b3 = take(O, (O,))
    return W1, b1, W2, b2, W3, b3


def forward(P, X, D, H, O):
    W1, b1, W2, b2, W3, b3 = unpack(P, D, H, O)
    X = np.asarray(X, dtype=np.float64)
    a1 = np.maximum(X @ W1.T + b1, 0.0)
    a2 = np.maximum(a1 @ W2.T + b2, 0.0)
    return a2 @ W3.T + b3, (X, a1, a2)


def loss_grad(P, X, T, D, H, O):
    W1, b1, W2, b2, W3, b3 = unpack(P, D, H, O)
    Y, (X, a1, a2) = forward(P, X, D, H, O)
    T = np.asarray(T, dtype=np.float64)
    n = X.shape[0]
    E = Y - T
    loss = float((E * E).sum() / (n * O))
    go = 2.0 * E / (n * O)
    g2 = (go @ W3) * (a2 > 0)
    g1 = (g2 @ W2) * (a1 > 0)
    grad = np.concatenate([(g1.T @ X).ravel(), g1.sum(0), (g2.T @ a1).ravel(), g2.sum(0),
                           (go.T @ a2).ravel(), go.sum(0)])
    return loss, grad
