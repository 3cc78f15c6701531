"""GPU solve against SuperLU with IFEM's options (SparseMatrix.C:101-104) on
the oracle's FP64 system, and the FP64-certified residual of the mixed
precision PCG."""
import numpy as np
import pytest

from ifem_gb300 import ifemgpu as G
from ifem_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def superlu_solution(orc):
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    s = orc.sizes
    A, b = orc.system()
    IA, JA = orc.pattern()
    K = sp.csc_matrix((A, JA, IA), shape=(s["neq"],) * 2)
    lu = sla.splu(K, permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.001,
                  options={"SymmetricMode": True})
    return lu.solve(b), K, b


def setup(patches, ng, ke=G.KE_FP64):
    import oracle
    sim = G.SIM(n_gauss=ng, ke_precision=ke)
    W.load_into(sim, patches)
    sim.preprocess()
    sim.assembleSystem()
    orc = oracle.OracleModel(ng)
    W.load_into(orc, patches)
    orc.preprocess()
    orc.assemble(8)
    return sim, orc


@pytest.mark.parametrize("method", [G.PCG_MIXED, G.PCG_FP64])
def test_config1_solution_matches_superlu(gpulib, oracle_lib, method):
    patches, ng = W.config1()
    sim, orc = setup(patches, ng)
    xref, K, b = superlu_solution(orc)
    x, info = sim.solveSystem(method=method, rtol=1e-12)
    assert info.relres <= 1e-12
    # FP64 residual of the GPU solution on the oracle's matrix
    assert np.linalg.norm(b - K @ x) / np.linalg.norm(b) <= 1e-11
    assert np.abs(x - xref).max() <= 1e-9 * np.abs(xref).max()
    u = sim.expand_solution(x)
    madof, meqn = orc.sam()
    np.testing.assert_array_equal(u[meqn == 0], 0.0)


def test_config2_small_elasticity_solution(gpulib, oracle_lib):
    patches, ng = W.config2(nel=6)
    sim, orc = setup(patches, ng)
    xref, K, b = superlu_solution(orc)
    x, info = sim.solveSystem(method=G.PCG_MIXED, rtol=1e-10)
    assert info.relres <= 1e-10
    assert np.linalg.norm(b - K @ x) / np.linalg.norm(b) <= 2e-10
    assert np.abs(x - xref).max() <= 1e-6 * np.abs(xref).max()


def test_iteration_cap_reports_not_converged(gpulib):
    patches, ng = W.config2(nel=6)
    sim = G.SIM(n_gauss=ng)
    W.load_into(sim, patches)
    sim.preprocess()
    sim.assembleSystem()
    x, info = sim.solveSystem(method=G.PCG_FP64, rtol=1e-12, max_inner=5, check=False)
    with pytest.raises(G.IfemGpuError) as e:
        sim.solveSystem(method=G.PCG_FP64, rtol=1e-12, max_inner=5)
    assert e.value.status == G.NOT_CONVERGED
    assert info.relres > 1e-12
