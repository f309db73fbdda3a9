"""Test-only numpy restatement of the learned branching scorer (the MLP of
gbx_scorer_forward and the listwise loss and gradient of gbx_scorer_gradient),
in float64, for gradient checks of the CUDA kernels. The scorer has no
counterpart in the reference; this file is the oracle for it.

Parameter layout: W1[H][F], b1[H], W2[H][H], b2[H], w3[H], b3.
"""
import numpy as np


def unpack(p, F, H):
    p = np.asarray(p, np.float64)
    o = 0
    W1 = p[o:o + H * F].reshape(H, F); o += H * F
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def forward(p, X, F, H):
    W1, b1, W2, b2, w3, b3 = unpack(p, F, H)
    X = np.asarray(X, np.float64)
    a1 = X @ W1.T + b1
    h1 = np.maximum(a1, 0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0)
    return h2 @ w3 + b3, (X, a1, h1, a2, h2)


def loss_and_grad(p, X, group_ptr, target, F, H):
    """L = sum_g -sum_r t_r log softmax_g(z)_r and dL/dp (same layout)."""
    W1, b1, W2, b2, w3, b3 = unpack(p, F, H)
    z, (X, a1, h1, a2, h2) = forward(p, X, F, H)
    t = np.asarray(target, np.float64)
    dz = np.zeros_like(z)
    L = 0.0
    for g in range(len(group_ptr) - 1):
        b, e = group_ptr[g], group_ptr[g + 1]
        zz = z[b:e]
        lse = zz.max() + np.log(np.exp(zz - zz.max()).sum())
        dz[b:e] = np.exp(zz - lse) - t[b:e]
        L -= (t[b:e] * (zz - lse)).sum()
    d2 = (dz[:, None] * w3[None, :]) * (a2 > 0)
    d1 = (d2 @ W2) * (a1 > 0)
    g = np.concatenate([(d1.T @ X).ravel(), d1.sum(0), (d2.T @ h1).ravel(), d2.sum(0), h2.T @ dz, [dz.sum()]])
    return L, g
