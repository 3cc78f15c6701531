"""TEST INFRASTRUCTURE ONLY: FP64 numpy restatement of the learned coarse
correction (network, loss, gradients and the coarse transfer), the checker of
the library's hand-written training kernels.

The reference (IFEM) has no counterpart: its solvers are SuperLU and
PETSc/ISTL Krylov methods.  Parity is pinned by finite differences of this
module's own loss (tests/test_oracle_mlp.py), not by reference vectors.

Parameter layout (one flat array, as ifemgpu_learn_get_weights returns it):
W1 (hidden x inputs, row-major), b1, W2 (hidden x hidden), b2,
W3 (outputs x hidden), b3.
"""
from __future__ import annotations

import numpy as np


def unpack(theta: np.ndarray, nin: int, nh: int, nout: int):
    o = 0
    W1 = theta[o:o + nh * nin].reshape(nh, nin); o += nh * nin
    b1 = theta[o:o + nh]; o += nh
    W2 = theta[o:o + nh * nh].reshape(nh, nh); o += nh * nh
    b2 = theta[o:o + nh]; o += nh
    W3 = theta[o:o + nout * nh].reshape(nout, nh); o += nout * nh
    b3 = theta[o:o + nout]; o += nout
    assert o == theta.size
    return W1, b1, W2, b2, W3, b3


def forward(theta, X, nh, nout):
    """Network outputs for the rows of X (ReLU after layers 1 and 2)."""
    W1, b1, W2, b2, W3, b3 = unpack(np.asarray(theta, np.float64), X.shape[1], nh, nout)
    X = np.asarray(X, np.float64)
    H1 = np.maximum(X @ W1.T + b1, 0.0)
    H2 = np.maximum(H1 @ W2.T + b2, 0.0)
    return H2 @ W3.T + b3, (X, H1, H2)


def loss_and_grad(theta, X, Y, nh):
    """mean((net(X) - Y)^2) and its gradient (flat, same layout as theta)."""
    nout = Y.shape[1]
    W1, b1, W2, b2, W3, b3 = unpack(np.asarray(theta, np.float64), X.shape[1], nh, nout)
    Yp, (X, H1, H2) = forward(theta, X, nh, nout)
    D = Yp - np.asarray(Y, np.float64)
    loss = float(np.mean(D * D))
    dY = 2.0 * D / D.size
    gW3 = dY.T @ H2
    gb3 = dY.sum(0)
    dH2 = (dY @ W3) * (H2 > 0)
    gW2 = dH2.T @ H1
    gb2 = dH2.sum(0)
    dH1 = (dH2 @ W2) * (H1 > 0)
    gW1 = dH1.T @ X
    gb1 = dH1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g


def greville(knots: np.ndarray, p: int) -> np.ndarray:
    n = len(knots) - p - 1
    return np.array([knots[i + 1:i + p + 1].mean() for i in range(n)])


def restriction(knots3, degree3, ncoef3, meqn, madof, npv: int, m: int):
    """Dense restriction R (npv (m+1)^3 x neq): trilinear weights of the
    coarse vertices at each free equation's Greville point (unit parameter
    cube after normalisation), rows ordered vertex-major, component-minor."""
    neq = int(meqn.max())
    gr = []
    for d in range(3):
        g = greville(np.asarray(knots3[d]), degree3[d])
        U = np.asarray(knots3[d])
        gr.append((g - U[degree3[d]]) / (U[ncoef3[d]] - U[degree3[d]]))
    nv = (m + 1) ** 3
    R = np.zeros((npv * nv, neq))
    n0, n1 = ncoef3[0], ncoef3[1]
    for node in range(int(np.prod(ncoef3))):
        i, j, k = node % n0, (node // n0) % n1, node // (n0 * n1)
        t = np.array([gr[0][i], gr[1][j], gr[2][k]]) * m
        c = np.clip(np.floor(t).astype(int), 0, m - 1)
        f = np.clip(t - c, 0.0, 1.0)
        for comp in range(npv):
            eq = meqn[madof[node] - 1 + comp]
            if eq <= 0:
                continue
            for dd in range(8):
                di, dj, dk = dd & 1, (dd >> 1) & 1, dd >> 2
                w = ((f[0] if di else 1 - f[0]) * (f[1] if dj else 1 - f[1])
                     * (f[2] if dk else 1 - f[2]))
                v = ((c[2] + dk) * (m + 1) + c[1] + dj) * (m + 1) + c[0] + di
                R[v * npv + comp, eq - 1] += w
    return R
