"""CPU checks of the FP64 Kronecker-preconditioner oracle (oracle/kron.py):
the fast-diagonalisation solve inverts the assembled Kronecker operator, and
the 1D spline matrices have the known row sums (partition of unity: the mass
rows sum to the basis integrals, stiffness rows of the full basis sum to 0)."""
import numpy as np

from oracle import kron


def knots(p, ne):
    return np.concatenate([np.zeros(p), np.linspace(0, 1, ne + 1), np.ones(p)])


def test_fast_diagonalisation_inverts_kronecker_operator():
    p = 3
    U = [knots(p, 4), knots(p, 5), knots(p, 3)]
    n = [len(u) - p - 1 for u in U]
    lo = [1, 1, 0]
    hi = [n[0] - 2, n[1] - 2, n[2] - 1]
    B = kron.KronBlock(U, [p, p, p], lo, hi)
    P = B.matrix()
    rng = np.random.default_rng(3)
    r = rng.standard_normal(P.shape[0])
    z = B.solve(r)
    assert np.abs(P @ z - r).max() <= 1e-10 * np.abs(r).max()
    assert np.allclose(B.diag(), np.diag(P))


def test_spline_matrices_row_sums():
    for p in (1, 2, 3):
        U = knots(p, 6)
        K, M = kron.matrices_1d(U, p)
        assert np.abs(K.sum(1)).max() <= 1e-12
        assert abs(M.sum() - 1.0) <= 1e-12
