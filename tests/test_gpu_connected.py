"""Conformingly connected patches on the GPU (ifemgpu_patch_connect),
through the C ABI: assembly against the oracle at sizes beyond the golden
systems (tests/test_gpu_ref_golden.py holds the IFEM-built ones), bitwise
reproducible assembly, and a solve across the patch interfaces."""
import numpy as np
import pytest

from ifem_gb300 import ifemgpu as G
from ifem_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def assemble(patches, ng, conns, ke):
    sim = G.SIM(n_gauss=ng, ke_precision=ke)
    W.load_into(sim, patches, conns)
    sim.preprocess()
    sim.assembleSystem()
    return sim


@pytest.mark.parametrize("kind", [1, 2], ids=["poisson", "elasticity"])
def test_connected_assembly_matches_oracle_and_repeats_bitwise(gpulib, oracle_lib, kind):
    import oracle
    patches, ng, conns = W.connected_boxes(kind, 2, 5, 3, rotated=True)
    sim = assemble(patches, ng, conns, G.KE_FP64)
    K, b = sim.matrix_values(), sim.rhs()
    orc = oracle.OracleModel(ng)
    W.load_into(orc, patches, conns)
    orc.preprocess()
    orc.assemble(8)
    Ko, bo = orc.system()
    IA, JA = orc.pattern()
    sam = sim.getSAM()
    np.testing.assert_array_equal(sam.colptr, IA)
    np.testing.assert_array_equal(sam.rowidx, JA)
    assert np.abs(K - Ko).max() <= 1e-12 * np.abs(Ko).max()
    assert np.abs(b - bo).max() <= 1e-12 * np.abs(bo).max()
    split = assemble(patches, ng, conns, G.KE_SPLIT_TF32)
    K1 = split.matrix_values()
    split.assembleSystem()
    assert np.array_equal(K1, split.matrix_values())       # deterministic
    assert np.abs(K1 - Ko).max() <= 5e-6 * np.abs(Ko).max()


def test_solve_across_interfaces(gpulib):
    patches, ng, conns = W.connected_boxes(1, 2, 6, 3, rotated=True)
    sim = assemble(patches, ng, conns, G.KE_SPLIT_TF32)
    x, info = sim.solveSystem(method=G.PCG_MIXED, rtol=1e-10)
    assert info.relres <= 1e-10
    u = sim.expand_solution(x)
    # the solution is continuous across interfaces by construction (shared
    # nodes); it is positive for a positive source with u = 0 on the ends
    assert u.min() >= -1e-12 and u.max() > 0
    with pytest.raises(G.IfemGpuError):     # Kronecker needs unconnected patches
        sim.solveSystem(method=G.PCG_MIXED, rtol=1e-10, precond=G.PRECOND_KRONECKER)
