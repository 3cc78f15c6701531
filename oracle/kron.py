"""TEST INFRASTRUCTURE ONLY: FP64 numpy restatement of the Kronecker-product
(fast-diagonalisation) preconditioner, the checker of the library's FD kernels.

The reference (IFEM) has no counterpart.  The method: on the box of free
control points of one patch component, P = K0xM1xM2 + M0xK1xM2 + M0xM1xK2
with the 1D spline stiffness K_d and mass M_d of the patch's knot vectors
(Gauss rule of p+1 points per span); P^-1 through the generalised
eigenproblems K_d U_d = M_d U_d diag(lam_d) (Lynch, Rice and Thomas 1964);
z = S P^-1 S r with S = sqrt(diag(P) / diag(A)).  Pinned by the identity
P P^-1 = I on a small case (tests/test_oracle_kron.py).
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla


def bspline_basis(U, p, x):
    """values and first derivatives of all B-splines of (U, p) at x
    (Cox-de Boor recursion on the full index range)."""
    U = np.asarray(U, dtype=np.float64)
    nb = len(U) - p - 1
    # degree-0 functions; the last non-empty span is closed on the right
    last = max(i for i in range(len(U) - 1) if U[i] < U[i + 1])
    N = np.array([1.0 if (U[i] <= x < U[i + 1]) or (i == last and x == U[i + 1]) else 0.0
                  for i in range(len(U) - 1)])
    Nprev = N
    for k in range(1, p + 1):
        Nk = np.zeros(len(U) - 1 - k)
        for i in range(len(Nk)):
            a = 0.0 if U[i + k] == U[i] else (x - U[i]) / (U[i + k] - U[i]) * Nprev[i]
            b = 0.0 if U[i + k + 1] == U[i + 1] else \
                (U[i + k + 1] - x) / (U[i + k + 1] - U[i + 1]) * Nprev[i + 1]
            Nk[i] = a + b
        if k == p:
            dN = np.zeros(nb)
            for i in range(nb):
                a = 0.0 if U[i + p] == U[i] else p / (U[i + p] - U[i]) * Nprev[i]
                b = 0.0 if U[i + p + 1] == U[i + 1] else p / (U[i + p + 1] - U[i + 1]) * Nprev[i + 1]
                dN[i] = a - b
        Nprev = Nk
    if p == 0:
        dN = np.zeros(nb)
    return Nprev[:nb], dN


def matrices_1d(U, p):
    U = np.asarray(U, dtype=np.float64)
    nb = len(U) - p - 1
    K = np.zeros((nb, nb))
    M = np.zeros((nb, nb))
    xg, wg = np.polynomial.legendre.leggauss(p + 1)
    kn = np.unique(U)
    for a, b in zip(kn[:-1], kn[1:]):
        for xq, wq in zip(xg, wg):
            x = 0.5 * (a + b) + 0.5 * (b - a) * xq
            w = 0.5 * (b - a) * wq
            N, dN = bspline_basis(U, p, x)
            K += w * np.outer(dN, dN)
            M += w * np.outer(N, N)
    return K, M


class KronBlock:
    """P^-1 on the box lo..hi (inclusive, per direction) of one component."""

    def __init__(self, knots3, degree3, lo, hi):
        self.K, self.M, self.U, self.lam = [], [], [], []
        for d in range(3):
            K, M = matrices_1d(knots3[d], degree3[d])
            sl = slice(lo[d], hi[d] + 1)
            K, M = K[sl, sl], M[sl, sl]
            lam, Uv = sla.eigh(K, M)
            self.K.append(K); self.M.append(M); self.U.append(Uv); self.lam.append(lam)
        self.n = [hi[d] - lo[d] + 1 for d in range(3)]

    def diag(self):
        """diagonal of P in box order (i fastest)"""
        dK = [np.diag(K) for K in self.K]
        dM = [np.diag(M) for M in self.M]
        return (dK[0][None, None, :] * dM[1][None, :, None] * dM[2][:, None, None]
                + dM[0][None, None, :] * dK[1][None, :, None] * dM[2][:, None, None]
                + dM[0][None, None, :] * dM[1][None, :, None] * dK[2][:, None, None]).ravel()

    def solve(self, r):
        """P^-1 r (r in box order, i fastest)"""
        U0, U1, U2 = self.U
        t = r.reshape(self.n[2], self.n[1], self.n[0])
        t = np.einsum('kji,ia,jb,kc->cba', t, U0, U1, U2)
        L = (self.lam[0][None, None, :] + self.lam[1][None, :, None] + self.lam[2][:, None, None])
        t = t / L
        return np.einsum('cba,ia,jb,kc->kji', t, U0, U1, U2).ravel()

    def matrix(self):
        K, M = self.K, self.M
        return (np.kron(M[2], np.kron(M[1], K[0])) + np.kron(M[2], np.kron(K[1], M[0]))
                + np.kron(K[2], np.kron(M[1], M[0])))


def apply(patch, meqn, madof, diagA, r, npv=1):
    """z = S P^-1 S r over the free DOFs of a one-patch model whose free
    DOFs of each component form a box of control points."""
    n = patch.ncoef
    z = np.zeros_like(r)
    for comp in range(npv):
        eqs = np.full(n[::-1], -1, dtype=np.int64)   # [k][j][i]
        for node in range(int(np.prod(n))):
            e = meqn[madof[node] - 1 + comp]
            if e > 0:
                i, j, k = node % n[0], (node // n[0]) % n[1], node // (n[0] * n[1])
                eqs[k, j, i] = e - 1
        free = np.argwhere(eqs >= 0)
        lo = free.min(0)[::-1]
        hi = free.max(0)[::-1]
        box = eqs[lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1].ravel()
        assert (box >= 0).all()
        B = KronBlock(patch.knots, patch.degree, lo, hi)
        s = np.sqrt(B.diag() / diagA[box])
        z[box] = s * B.solve(s * r[box])
    return z
