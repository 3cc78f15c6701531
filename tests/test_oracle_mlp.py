"""CPU checks of the FP64 network oracle (oracle/mlp.py): its analytic
gradient against central finite differences of its own loss.  The reference
has no learned component, so this pins the oracle that the GPU training
kernels are compared with."""
import numpy as np

from oracle import mlp


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(5)
    nin, nh, nout, n = 7, 5, 4, 9
    npar = nh * nin + nh + nh * nh + nh + nout * nh + nout
    theta = rng.standard_normal(npar) * 0.5
    X = rng.standard_normal((n, nin))
    Y = rng.standard_normal((n, nout))
    loss, g = mlp.loss_and_grad(theta, X, Y, nh)
    h = 1e-6
    fd = np.zeros(npar)
    for i in range(npar):
        tp = theta.copy(); tp[i] += h
        tm = theta.copy(); tm[i] -= h
        fd[i] = (mlp.loss_and_grad(tp, X, Y, nh)[0] - mlp.loss_and_grad(tm, X, Y, nh)[0]) / (2 * h)
    assert np.abs(g - fd).max() <= 1e-7 * max(1.0, np.abs(fd).max())
    assert loss > 0


def test_oracle_restriction_partition_of_unity():
    # trilinear weights of each free equation sum to one over the coarse vertices
    p, ne, m = 3, 6, 2
    U = np.concatenate([np.zeros(p), np.linspace(0, 1, ne + 1), np.ones(p)])
    n = ne + p
    madof = np.arange(1, n ** 3 + 2, dtype=np.int32)
    meqn = np.arange(1, n ** 3 + 1, dtype=np.int32)
    R = mlp.restriction([U, U, U], [p, p, p], [n, n, n], meqn, madof, 1, m)
    assert R.shape == ((m + 1) ** 3, n ** 3)
    assert np.allclose(R.sum(0), 1.0)
