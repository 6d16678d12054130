"""FP64 numpy restatement of the engine-switch MLP (forward, weighted BCE loss, gradients).

TEST INFRASTRUCTURE ONLY: the GPU forward/backward kernels of
grazelle-ppopp18_gb300/csrc/grz_switch.cu are checked against it.  The parameter layout is
the kernels': W1[H][F] b1[H] W2[H][H] b2[H] W3[H] b3.
"""
from __future__ import annotations

import numpy as np

F, H = 12, 32
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * F
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H
NP = OFF_B3 + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    W1 = p[OFF_W1:OFF_B1].reshape(H, F)
    b1 = p[OFF_B1:OFF_W2]
    W2 = p[OFF_W2:OFF_B2].reshape(H, H)
    b2 = p[OFF_B2:OFF_W3]
    W3 = p[OFF_W3:OFF_B3]
    b3 = p[OFF_B3]
    return W1, b1, W2, b2, W3, b3


def forward(p, X):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    a1 = X @ W1.T + b1
    h1 = np.maximum(a1, 0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0)
    z = h2 @ W3 + b3
    return z, (X, a1, h1, a2, h2)


def loss_and_grad(p, X, Y, W):
    """mean over samples of W * (softplus(z) - Y z), and its gradient w.r.t. the parameters."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    z, (X, a1, h1, a2, h2) = forward(p, X)
    Y = np.asarray(Y, dtype=np.float64)
    Wt = np.asarray(W, dtype=np.float64)
    n = X.shape[0]
    softplus = np.logaddexp(0.0, z)
    loss = float(np.sum(Wt * (softplus - Y * z)) / n)
    dz = Wt * (0.5 * (1.0 + np.tanh(0.5 * z)) - Y)
    g = np.zeros(NP)
    g[OFF_B3] = dz.sum()
    g[OFF_W3:OFF_B3] = h2.T @ dz
    dh2 = np.outer(dz, W3) * (a2 > 0)
    g[OFF_B2:OFF_W3] = dh2.sum(0)
    g[OFF_W2:OFF_B2] = (dh2.T @ h1).reshape(-1)
    dh1 = (dh2 @ W2) * (a1 > 0)
    g[OFF_B1:OFF_W2] = dh1.sum(0)
    g[OFF_W1:OFF_B1] = (dh1.T @ X).reshape(-1)
    return loss, g / n
