"""Solution norms and secondary solution on the GPU, through the C ABI:
against the FP64 oracle (tests/test_oracle_norms.py pins the oracle to closed
forms), and a(u, u) = x^T K x of the assembled system at a size beyond the
oracle's reach."""
import numpy as np
import pytest

from ifem_gb300 import ifemgpu as G
from ifem_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def both(patches, ng, ke):
    import oracle
    sim = G.SIM(n_gauss=ng, ke_precision=ke)
    W.load_into(sim, patches)
    sim.preprocess()
    sim.assembleSystem()
    orc = oracle.OracleModel(ng)
    W.load_into(orc, patches)
    orc.preprocess()
    return sim, orc


@pytest.mark.parametrize("ke,tol", [(G.KE_FP64, 1e-11), (G.KE_SPLIT_TF32, 2e-5)],
                         ids=["fp64", "split"])
@pytest.mark.parametrize("case", ["poisson_p3_kappa", "elasticity_nurbs"])
def test_norms_and_secondary_match_oracle(gpulib, oracle_lib, case, ke, tol):
    if case == "poisson_p3_kappa":
        patches, ng = W.config4(nel=4, grid=16)
        nq, nc = 64, 3
    else:
        patches, ng = W.config2(nel=3)
        nq, nc = 27, 6
    sim, orc = both(patches, ng, ke)
    u = np.random.default_rng(5).standard_normal(sim.sizes.ndof)
    tot, el = sim.solution_norms(u, per_element=True)
    tot_o, el_o = orc.norms(u, per_element=True)
    assert np.abs(tot - tot_o).max() <= tol * np.abs(tot_o).max()
    assert np.abs(el - el_o).max() <= tol * np.abs(el_o).max()
    sec = sim.secondary_solution(1, u, nq, nc)
    sec_o = orc.secondary(1, u, patches[0].nel, nq, nc)
    assert np.abs(sec - sec_o).max() <= 10 * tol * np.abs(sec_o).max()


@pytest.mark.parametrize("ke,tol", [(G.KE_FP64, 1e-10), (G.KE_SPLIT_TF32, 2e-5)],
                         ids=["fp64", "split"])
def test_energy_norm_equals_xKx(gpulib, ke, tol):
    patches, ng = W.config4(nel=24)
    sim = G.SIM(n_gauss=ng, ke_precision=ke)
    W.load_into(sim, patches)
    sim.preprocess()
    sim.assembleSystem()
    x, info = sim.solveSystem(method=G.PCG_FP64 if ke == G.KE_FP64 else G.PCG_MIXED, rtol=1e-10)
    K = sim.matrix_values()
    sam = sim.getSAM()
    n = len(sam.colptr) - 1
    cols = np.repeat(np.arange(n), np.diff(sam.colptr))
    Kx = np.zeros(n)
    np.add.at(Kx, sam.rowidx, K * x[cols])
    xKx = float(x @ Kx)
    energy, _ = sim.solution_norms(sim.expand_solution(x))
    assert abs(energy - xKx) <= tol * xKx
    # with homogeneous Dirichlet conditions a(u, u) = b^T x as well
    assert abs(energy - float(sim.rhs() @ x)) <= max(tol, 1e-9) * xKx
