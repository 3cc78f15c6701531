"""Kronecker (fast-diagonalisation) preconditioner kernels against the FP64
numpy oracle (oracle/kron.py), through ifemgpu_apply_preconditioner: the
Poisson patch of the log-normal conductivity family (p = 3, all faces
fixed) and the elasticity patch (p = 2, one face clamped, three components).
FP32 kernels: 2e-5 of the largest entry."""
import numpy as np
import pytest

from ifem_gb300 import ifemgpu as G
from ifem_gb300 import workloads as W
from oracle import kron

pytestmark = pytest.mark.gpu


def diagonal(sim):
    sam = sim.getSAM()
    vals = sim.matrix_values()
    d = np.zeros(sim.sizes.neq)
    for j in range(sim.sizes.neq):
        rows = sam.rowidx[sam.colptr[j]:sam.colptr[j + 1]]
        d[j] = vals[sam.colptr[j] + np.searchsorted(rows, j)]
    return d


@pytest.mark.parametrize("case", ["poisson_p3", "elasticity_p2"])
def test_kronecker_apply_matches_oracle(gpulib, case):
    if case == "poisson_p3":
        patches, ng = W.config4(nel=7, p=3)
        npv = 1
    else:
        patches, ng = W.config2(nel=5, p=2)
        npv = 3
    sim = G.SIM(n_gauss=ng, ke_precision=G.KE_FP64)
    W.load_into(sim, patches)
    sim.preprocess()
    sim.assembleSystem()
    sam = sim.getSAM()
    rng = np.random.default_rng(8)
    r = rng.standard_normal(sim.sizes.neq)
    z = sim.apply_preconditioner(r, G.PRECOND_KRONECKER)
    ref = kron.apply(patches[0], sam.meqn, sam.madof, diagonal(sim), r, npv=npv)
    assert np.abs(z - ref).max() <= 2e-5 * np.abs(ref).max()
    zj = sim.apply_preconditioner(r, G.PRECOND_JACOBI)
    assert np.abs(zj - r / diagonal(sim)).max() <= 1e-6 * np.abs(zj).max()
