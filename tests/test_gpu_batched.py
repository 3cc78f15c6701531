"""Batched multi-patch assembly (64 independent patches of uneven size and
degree, Poisson and elasticity integrands): one system per integrand type,
as two IFEM simulators would number them, each assembled by one persistent
colour-major launch of the generic element kernel, or in split precision one
launch per tensor-core kernel (p = 2 elasticity, p = 2 and p = 3 Poisson)
plus the generic launch for the rest.

- FP64 mode against the oracle (relative 1e-12);
- the persistent launch gives the same bits as one launch per colour (the
  per-entry summation order is the colour order in both);
- repeated assemblies are bitwise identical, with the autotuned tiles;
- the block-CSR copy of the elasticity system holds the same matrix;
- the full 64-patch configuration: persistent == colour passes, and the
  launch count of one assembly.
"""
import numpy as np
import pytest

from ifem_gb300 import ifemgpu as G
from ifem_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def by_kind(patches, kind):
    return [pc for pc in patches if pc.kind == kind]


def assemble(patches, ng, ke, colour_passes=0):
    sim = G.SIM(n_gauss=ng, ke_precision=ke, colour_passes=colour_passes)
    W.load_into(sim, patches)
    sim.preprocess()
    sim.assembleSystem()
    return sim, sim.matrix_values(), sim.rhs()


@pytest.mark.parametrize("kind", [1, 2])
def test_two_systems_match_oracle_fp64(gpulib, oracle_lib, kind):
    import oracle
    patches, ng = W.config3(npatch=12, nmin=2, nmax=5)
    sub = by_kind(patches, kind)
    assert sub
    sim, K, b = assemble(sub, ng, G.KE_FP64)
    orc = oracle.OracleModel(ng)
    W.load_into(orc, sub)
    orc.preprocess()
    orc.assemble(8)
    Ko, bo = orc.system()
    IA, JA = orc.pattern()
    sam = sim.getSAM()
    np.testing.assert_array_equal(sam.colptr, IA)
    np.testing.assert_array_equal(sam.rowidx, JA)
    assert np.abs(K - Ko).max() <= 1e-12 * np.abs(Ko).max()
    assert np.abs(b - bo).max() <= 1e-12 * np.abs(bo).max()


@pytest.mark.parametrize("ke", [G.KE_FP64, G.KE_SPLIT_TF32])
@pytest.mark.parametrize("kind", [1, 2])
def test_persistent_launch_equals_colour_passes(gpulib, ke, kind):
    patches, ng = W.config3(npatch=16, nmin=3, nmax=7)
    sub = by_kind(patches, kind)
    s1, K1, b1 = assemble(sub, ng, ke, colour_passes=2)
    s2, K2, b2 = assemble(sub, ng, ke, colour_passes=1)
    assert np.array_equal(K1, K2) and np.array_equal(b1, b2)
    s1.assembleSystem()
    assert np.array_equal(s1.matrix_values(), K1) and np.array_equal(s1.rhs(), b1)
    s1.assembly_stats()
    s2.assembly_stats()
    if ke == G.KE_SPLIT_TF32:  # every patch on the tensor-core kernels (p = 2 and 3)
        assert s1.kernel_launches == s2.kernel_launches
        assert s1.kernel_launches <= 5  # basis tables, one element kernel and one gather per degree
    else:
        assert s1.kernel_launches < s2.kernel_launches


def test_block_csr_copy(gpulib):
    patches, ng = W.config3(npatch=8, nmin=2, nmax=4)
    sub = by_kind(patches, 2)
    for pc in sub:                       # clamp whole nodes only
        pc.dirichlet = [(5, 123, 0.0)]
    sim, K, b = assemble(sub, ng, G.KE_FP64)
    rp, ci, blocks = sim.matrix_bsr(3)
    sam = sim.getSAM()
    n = sim.sizes.neq
    import scipy.sparse as sp
    A = sp.csc_matrix((K, sam.rowidx, sam.colptr), shape=(n, n)).toarray()
    B = sp.bsr_matrix((blocks, ci, rp), shape=(n, n)).toarray()
    assert np.array_equal(A, B)


def test_full_config3_persistent(gpulib):
    patches, ng = W.config3()
    for kind in (1, 2):
        sub = by_kind(patches, kind)
        s1, K1, b1 = assemble(sub, ng, G.KE_SPLIT_TF32, colour_passes=2)
        s2, K2, b2 = assemble(sub, ng, G.KE_SPLIT_TF32, colour_passes=1)
        s3, K3, b3 = assemble(sub, ng, G.KE_SPLIT_TF32, colour_passes=0)
        assert np.array_equal(K1, K2) and np.array_equal(b1, b2)
        assert np.array_equal(K1, K3) and np.array_equal(b1, b3)
        t1, v1, _ = s1.assembly_stats()
        t2, v2, _ = s2.assembly_stats()
        t3, v3, _ = s3.assembly_stats()
        print(f"\nconfig 3 kind {kind}: {len(sub)} patches, {s1.sizes.nel} elements, "
              f"persistent {t1:.2f} ms ({s1.kernel_launches} launches), "
              f"colour passes {t2:.2f} ms ({s2.kernel_launches} launches), "
              f"autotuned {t3:.2f} ms ({s3.kernel_launches} launches)")
        assert s3.kernel_launches <= 5   # one element launch and one gather per degree
