"""Consistent mass matrix added to the stiffness (K + s M, the effective
stiffness of implicit time stepping), through the C ABI.

Against IFEM's own Weak::Mass assembly the golden systems c6/c7 of
tests/golden/ref_systems.npz cover it (tests/test_gpu_ref_golden.py); here
size-independent properties at sizes beyond the oracle's reach:
linearity in s, M = (K(s) - K(0)) / s symmetric and non-negative (B-spline
bases are non-negative), and the sum of all entries of M equal to the volume
of the domain (partition of unity) -- per component for elasticity.
"""
import numpy as np
import pytest

from ifem_gb300 import ifemgpu as G
from ifem_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def assemble(patch, ng, mass, ke=G.KE_FP64):
    patch.mass = mass
    sim = G.SIM(n_gauss=ng, ke_precision=ke)
    W.load_into(sim, [patch])
    sim.preprocess()
    sim.assembleSystem()
    return sim, sim.matrix_values()


@pytest.mark.parametrize("kind,nel,ke,tol", [(1, 16, G.KE_FP64, 1e-12), (1, 16, G.KE_SPLIT_TF32, 2e-6),
                                             (2, 8, G.KE_FP64, 1e-12), (2, 8, G.KE_SPLIT_TF32, 2e-6)])
def test_mass_is_linear_symmetric_and_integrates_the_volume(gpulib, kind, nel, ke, tol):
    pc = W.box_patch(3, 2, nel, size=(1.0, 2.0, 0.5))     # volume 1, no Dirichlet DOFs
    pc.kind = kind
    _, K0 = assemble(pc, 3, 0.0, ke)
    sim, K1 = assemble(pc, 3, 3.0, ke)
    _, K2 = assemble(pc, 3, 6.0, ke)
    M = (K1 - K0) / 3.0
    scale = np.abs(K2).max()
    assert np.abs((K2 - K0) - 2.0 * (K1 - K0)).max() <= 10 * tol * scale
    sam = sim.getSAM()
    n = len(sam.colptr) - 1
    cols = np.repeat(np.arange(n), np.diff(sam.colptr))
    rows = sam.rowidx
    # symmetric: entry (i, j) equals (j, i)
    key = rows.astype(np.int64) * n + cols
    tkey = cols.astype(np.int64) * n + rows
    order = np.argsort(key)
    pos = order[np.searchsorted(key[order], tkey)]
    assert np.abs(M - M[pos]).max() <= 10 * tol * scale
    assert M.min() >= -10 * tol * scale
    ncomp = 1 if kind == 1 else 3
    assert abs(M.sum() - ncomp * 1.0) <= 1e3 * tol * ncomp
