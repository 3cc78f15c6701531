"""Tensor-core (tcgen05, 3xTF32) element path against FP64 references.

Tolerances: the split-precision element matrices carry ~1e-6 relative
error (TF32 split products, FP32 accumulation); the assembled matrix is
compared in max norm, 5e-6 of max|K|, and entry by entry for entries above
1e-3 of max|K| at 1e-4 relative.  The FP64 scatter keeps the assembly
deterministic (two runs bit-identical)."""
import numpy as np
import pytest

from ifem_gb300 import ifemgpu as G
from ifem_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TC_TOL = 5e-6


def test_selftest_gemm_3xtf32(gpulib):
    rng = np.random.default_rng(7)
    A = rng.standard_normal((128, 32)).astype(np.float32)
    B = rng.standard_normal((96, 32)).astype(np.float32)
    D = G.selftest_tc_gemm(A, B)
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    err = np.abs(D - ref).max() / np.abs(ref).max()
    assert err < 2e-6, err


def test_selftest_gemm_layout_rows_and_columns(gpulib):
    """Unit vectors locate every row/column/K index: D = A B^T with A, B
    permutation-like patterns must be reproduced exactly."""
    A = np.zeros((128, 32), np.float32)
    B = np.zeros((96, 32), np.float32)
    for r in range(128):
        A[r, r % 32] = r + 1
    for c in range(96):
        B[c, (c * 7) % 32] = 1.0 + c / 128
    D = G.selftest_tc_gemm(A, B)
    ref = (A.astype(np.float64) @ B.astype(np.float64).T)
    np.testing.assert_allclose(D, ref, rtol=1e-6, atol=0)


def assemble(patches, ng, ke):
    sim = G.SIM(n_gauss=ng, ke_precision=ke)
    W.load_into(sim, patches)
    sim.preprocess()
    sim.assembleSystem()
    return sim, sim.matrix_values(), sim.rhs()


@pytest.mark.parametrize("nel", [4, 12, 24])
def test_split_elasticity_vs_oracle(gpulib, oracle_lib, nel):
    import oracle
    patches, ng = W.config2(nel=nel)
    patches[0].body = (0.0, 0.5, -1.0)
    sim, K, b = assemble(patches, ng, G.KE_SPLIT_TF32)
    orc = oracle.OracleModel(ng)
    W.load_into(orc, patches)
    orc.preprocess()
    orc.assemble(8)
    Ko, bo = orc.system()
    scale = np.abs(Ko).max()
    err = np.abs(K - Ko).max() / scale
    assert err < TC_TOL, err
    big = np.abs(Ko) > 1e-3 * scale
    per = np.abs(K[big] - Ko[big]) / np.abs(Ko[big])
    assert per.max() < 1e-4, per.max()
    assert np.abs(b - bo).max() / np.abs(bo).max() < TC_TOL
    _, _, singular = sim.assembly_stats()
    assert singular == 0
    assert_exactly_symmetric(sim, K)


def test_split_assembly_deterministic(gpulib):
    patches, ng = W.config2(nel=12)
    sim, K1, b1 = assemble(patches, ng, G.KE_SPLIT_TF32)
    sim.assembleSystem()
    K2, b2 = sim.matrix_values(), sim.rhs()
    assert np.array_equal(K1, K2) and np.array_equal(b1, b2)


def test_split_assembly_solves_to_fp64_residual(gpulib):
    patches, ng = W.config2(nel=12)
    sim, K, b = assemble(patches, ng, G.KE_SPLIT_TF32)
    x, info = sim.solveSystem(method=G.PCG_MIXED, rtol=1e-10)
    assert info.relres <= 1e-10


def assert_exactly_symmetric(sim, K):
    """IFEM's element matrices are symmetric bit for bit, and the solvers
    take the compressed-column arrays row-wise: so must ours be."""
    import scipy.sparse as sp
    sam = sim.getSAM()
    A = sp.csc_matrix((K, sam.rowidx, sam.colptr), shape=(sim.sizes.neq,) * 2)
    assert (A - A.T).count_nonzero() == 0 or abs(A - A.T).max() == 0.0


def split_vs_oracle(patches, ng, tol=TC_TOL):
    import oracle
    sim, K, b = assemble(patches, ng, G.KE_SPLIT_TF32)
    orc = oracle.OracleModel(ng)
    W.load_into(orc, patches)
    orc.preprocess()
    orc.assemble(8)
    Ko, bo = orc.system()
    err = np.abs(K - Ko).max() / np.abs(Ko).max()
    assert err < tol, err
    if np.abs(bo).max() > 0:
        assert np.abs(b - bo).max() / np.abs(bo).max() < tol
    return sim, orc


def test_split_poisson2d_config1(gpulib, oracle_lib):
    split_vs_oracle(*W.config1())


def test_split_poisson3d_p3_kappa_field(gpulib, oracle_lib):
    split_vs_oracle(*W.config4(nel=6, grid=16))


@pytest.mark.parametrize("p", [2, 3])
def test_split_poisson3d_tensor_core_kernel(gpulib, oracle_lib, p):
    """p = 2 and 3 Poisson patches run on the tensor-core Poisson kernel:
    rational geometry, log-conductivity field, sine source with nodal noise
    and a prescribed non-zero face value (right-hand side corrections), even
    with colour passes forced for the generic kernel (one volume launch)."""
    import oracle
    rng = np.random.default_rng(77 + p)
    pc = W.perturb(W.box_patch(3, p, 5), rng, 0.1)
    pc.kind = 1
    pc.source, pc.source_shape = 2.0, 1
    pc.noise = 0.1 * rng.standard_normal(pc.nnod)
    pc.log_kappa = W.gaussian_field_3d(rng, pc.coefs[:, :3], grid=16)
    pc.dirichlet = [(1, 1, 0.5), (2, 1, 0.0), (5, 1, 0.0)]
    sim = G.SIM(n_gauss=0, ke_precision=G.KE_SPLIT_TF32, colour_passes=1)
    W.load_into(sim, [pc])
    sim.preprocess()
    sim.assembleSystem()
    K, b = sim.matrix_values(), sim.rhs()
    orc = oracle.OracleModel(0)
    W.load_into(orc, [pc])
    orc.preprocess()
    orc.assemble(8)
    Ko, bo = orc.system()
    scale = np.abs(Ko).max()
    assert np.abs(K - Ko).max() / scale < TC_TOL
    big = np.abs(Ko) > 1e-3 * scale
    assert (np.abs(K[big] - Ko[big]) / np.abs(Ko[big])).max() < 1e-4
    assert np.abs(b - bo).max() / np.abs(bo).max() < TC_TOL
    _, _, singular = sim.assembly_stats()
    assert singular == 0
    assert sim.kernel_launches <= 4     # basis tables + one element launch (not p^3 colours)
    assert_exactly_symmetric(sim, K)
    sim.assembleSystem()
    assert np.array_equal(sim.matrix_values(), K) and np.array_equal(sim.rhs(), b)


@pytest.mark.parametrize("kind,p", [(2, 2), (1, 2), (1, 3)])
def test_split_folded_geometry(gpulib, oracle_lib, kind, p):
    """An interior control point pushed past its neighbour folds the map: some
    |J| w turn negative (IFEM integrates them with their sign), which the
    tensor-core kernels integrate in a second pass with the MMA's negate-A
    bit.  Entries partly cancel, so the comparison is in max norm only."""
    import oracle
    pc = W.box_patch(3, p, 4)
    n0, n1, _ = pc.ncoef
    node = (2 * n1 + 2) * n0 + 2
    pc.coefs = pc.coefs.copy()
    pc.coefs[node, 0] += 0.45       # past the next control point in x
    pc.kind = kind
    if kind == 1:
        pc.source = 1.0
        pc.dirichlet = [(1, 1, 0.0), (2, 1, 0.0)]
    else:
        pc.dirichlet = [(5, 123, 0.0)]
        pc.neumann = [(6, (0.0, 0.0, 1.0))]
    sim = G.SIM(n_gauss=0, ke_precision=G.KE_SPLIT_TF32, colour_passes=1)
    W.load_into(sim, [pc])
    sim.preprocess()
    sim.assembleSystem()
    K, b = sim.matrix_values(), sim.rhs()
    sim.assembly_stats()
    assert sim.kernel_launches <= 4              # the tensor-core kernel took the patch
    orc = oracle.OracleModel(0)
    W.load_into(orc, [pc])
    orc.preprocess()
    orc.assemble(8)
    Ko, bo = orc.system()
    assert np.abs(K - Ko).max() / np.abs(Ko).max() < TC_TOL
    assert np.abs(b - bo).max() / np.abs(bo).max() < TC_TOL
    assert_exactly_symmetric(sim, K)


def test_split_multipatch_mixed(gpulib, oracle_lib):
    patches, ng = W.config3(npatch=6, nmin=2, nmax=5)
    split_vs_oracle(patches, ng)


@pytest.mark.parametrize("nel", [3, 6])
def test_split_elasticity_p3_tensor_core(gpulib, oracle_lib, nel):
    """p=3 elasticity (192 DOFs per element) on its tensor-core kernel: two
    MMA blocks (rows 0..127 x 192, rows 128..191 x 64), the element block
    mirrored from the upper triangle, with the traction face and a body
    force; basis tables, element kernel and gather are the only launches."""
    patches, _ = W.config2(nel=nel, p=3)
    patches[0].body = (0.2, 0.0, -0.5)
    sim, orc = split_vs_oracle(patches, 0)      # nGauss 0: p + 1 = 4 points per direction
    K = sim.matrix_values()
    big = np.abs(K) > 1e-3 * np.abs(K).max()
    Ko, _ = orc.system()
    assert (np.abs(K[big] - Ko[big]) / np.abs(Ko[big])).max() < 1e-4
    _, _, singular = sim.assembly_stats()
    assert singular == 0
    assert sim.kernel_launches <= 3
    assert_exactly_symmetric(sim, K)
    sim.assembleSystem()
    assert np.array_equal(sim.matrix_values(), K)


def test_config4_family_solve_matches_direct(gpulib, oracle_lib):
    import oracle
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    patches, ng = W.config4(nel=10, grid=16)
    sim, K, b = assemble(patches, ng, G.KE_SPLIT_TF32)
    x, info = sim.solveSystem(method=G.PCG_MIXED, rtol=1e-10)
    assert info.relres <= 1e-10
    sam = sim.getSAM()
    Km = sp.csc_matrix((K, sam.rowidx, sam.colptr), shape=(sim.sizes.neq,) * 2)
    # certified in FP64 on the assembled system
    assert np.linalg.norm(b - Km @ x) / np.linalg.norm(b) <= 1.5e-10
    orc = oracle.OracleModel(ng)
    W.load_into(orc, patches)
    orc.preprocess()
    orc.assemble(8)
    Ko, bo = orc.system()
    Kmo = sp.csc_matrix((Ko, sam.rowidx, sam.colptr), shape=(sim.sizes.neq,) * 2)
    xo = sla.spsolve(Kmo, bo)
    assert np.abs(x - xo).max() <= 1e-5 * np.abs(xo).max()


def test_assembly_phase_timings(gpulib):
    """The element-kernel and gather phases of a tensor-core assembly are
    timed by events between their captured segments: both positive, and
    together the volume time of the assembly statistics."""
    patches, ng = W.config2(nel=12)
    sim = G.SIM(n_gauss=ng, ke_precision=G.KE_SPLIT_TF32)
    W.load_into(sim, patches)
    sim.preprocess()
    for _ in range(2):
        sim.assembleSystem()
    total, volume, _ = sim.assembly_stats()
    elem, gath = sim.assembly_phases()
    assert sim.kernel_launches == 3          # basis tables, element kernel, gather
    assert elem > 0.0 and gath > 0.0
    assert abs((elem + gath) - volume) <= 1e-3 * volume + 1e-3
    assert volume <= total
