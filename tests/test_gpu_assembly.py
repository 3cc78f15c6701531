"""GPU assembly parity against the CPU oracle, through the C ABI.

FP64 element arithmetic (IFEMGPU_KE_FP64) must reproduce the oracle's K and b
to 1e-12 relative (max-norm over the matrix; per entry above 1e-9 of the
max), with the pattern bit-exact.  Sizes are chosen so that the oracle runs
in seconds.
"""
import numpy as np
import pytest

from ifem_gb300 import ifemgpu as G
from ifem_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def assemble_both(patches, ng, ke=G.KE_FP64, threads=8):
    import oracle
    sim = G.SIM(n_gauss=ng, ke_precision=ke)
    W.load_into(sim, patches)
    sim.preprocess()
    sim.assembleSystem()
    K, b = sim.matrix_values(), sim.rhs()
    orc = oracle.OracleModel(ng)
    W.load_into(orc, patches)
    orc.preprocess()
    orc.assemble(threads)
    Ko, bo = orc.system()
    sam = sim.getSAM()
    IA, JA = orc.pattern()
    np.testing.assert_array_equal(sam.colptr, IA)
    np.testing.assert_array_equal(sam.rowidx, JA)
    return sim, orc, K, b, Ko, bo


def rel_err(a, ref):
    scale = max(np.abs(ref).max(), 1e-300)
    return np.abs(a - ref).max() / scale


def check_fp64(K, b, Ko, bo, tol=FP64_TOL):
    assert rel_err(K, Ko) <= tol, rel_err(K, Ko)
    if np.abs(bo).max() > 0:
        assert rel_err(b, bo) <= tol, rel_err(b, bo)
    # entry by entry: entries formed by cancellation carry an absolute error
    # of the size of their largest element contribution, hence the floor
    big = np.abs(Ko) > 1e-6 * np.abs(Ko).max()
    per = np.abs(K[big] - Ko[big]) / np.abs(Ko[big])
    assert per.max() <= 1e4 * tol, per.max()


def test_config1_poisson2d_fp64(gpulib, oracle_lib):
    patches, ng = W.config1()
    sim, orc, K, b, Ko, bo = assemble_both(patches, ng)
    check_fp64(K, b, Ko, bo)
    _, _, singular = sim.assembly_stats()
    assert singular == 0


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_poisson2d_degrees(gpulib, oracle_lib, p):
    patches, ng = W.config1(nel=6, p=p)
    check_fp64(*assemble_both(patches, 0)[2:])


def test_config2_elasticity_nurbs_fp64_small(gpulib, oracle_lib):
    patches, ng = W.config2(nel=6)
    check_fp64(*assemble_both(patches, ng)[2:])


def test_config2_elasticity_nurbs_fp64_full(gpulib, oracle_lib):
    patches, ng = W.config2()
    check_fp64(*assemble_both(patches, ng)[2:])


def test_poisson3d_p3_kappa_field(gpulib, oracle_lib):
    patches, ng = W.config4(nel=6, grid=16)
    check_fp64(*assemble_both(patches, ng)[2:])


def test_elasticity_p3_body_force_and_traction(gpulib, oracle_lib):
    patches, ng = W.config2(nel=3, p=3)
    patches[0].body = (0.1, -0.2, 0.3)
    patches[0].neumann = [(6, (0.0, 0.0, 1.0)), (2, (0.5, 0.0, -0.25))]
    check_fp64(*assemble_both(patches, 0)[2:])


def test_prescribed_dirichlet_rhs(gpulib, oracle_lib):
    """Inhomogeneous Dirichlet values enter b as -c0 K(i,j) (assemSparse,
    src/LinAlg/SparseMatrix.C:639-687)."""
    patches, ng = W.config2(nel=4)
    patches[0].dirichlet = [(5, 123, 0.0), (6, 3, 0.01), (1, 1, -0.02)]
    patches[0].neumann = []
    sim, orc, K, b, Ko, bo = assemble_both(patches, ng)
    assert sim.sizes.nceq > 0
    check_fp64(K, b, Ko, bo)


def test_multi_patch_mixed(gpulib, oracle_lib):
    patches, ng = W.config3(npatch=6, nmin=2, nmax=5)
    check_fp64(*assemble_both(patches, ng)[2:])


def test_assembly_is_deterministic(gpulib):
    patches, ng = W.config2(nel=8)
    sim = G.SIM(n_gauss=ng)
    W.load_into(sim, patches)
    sim.preprocess()
    sim.assembleSystem()
    K1, b1 = sim.matrix_values(), sim.rhs()
    sim.assembleSystem()
    K2, b2 = sim.matrix_values(), sim.rhs()
    assert np.array_equal(K1, K2) and np.array_equal(b1, b2)


def test_singular_points_are_counted_and_skipped(gpulib, oracle_lib):
    """Collinear control points give det J = 0 exactly at every point; IFEM
    skips such points (src/ASM/ASMs3D.C:2286) and so does the GPU path."""
    patches, ng = W.config1(nel=3)
    pc = patches[0]
    pc.coefs[:, 1] = pc.coefs[:, 0]
    sim, orc, K, b, Ko, bo = assemble_both(patches, ng, threads=1)
    _, _, singular = sim.assembly_stats()
    assert singular == 9 * 9
    assert not K.any() and not b.any() and not Ko.any()


def test_matrix_copy_into_pinned_and_pageable_memory(gpulib):
    """ifemgpu_copy_matrix into pinned and pageable host memory, aligned or
    not: the same bits."""
    torch = pytest.importorskip("torch")
    patches, ng = W.config2(nel=6)
    sim = G.SIM(n_gauss=ng, ke_precision=G.KE_SPLIT_TF32)
    W.load_into(sim, patches)
    sim.preprocess()
    sim.assembleSystem()
    nnz = sim.sizes.nnz
    pageable = np.empty(nnz + 1, dtype=np.float64)
    sim.copy_matrix_into(pageable)
    pinned = torch.empty(nnz + 1, dtype=torch.float64).pin_memory().numpy()
    sim.copy_matrix_into(pinned)
    assert np.array_equal(pinned[:nnz], pageable[:nnz])
    odd = torch.empty(nnz + 1, dtype=torch.float64).pin_memory().numpy()[1:]   # 8-byte aligned only
    sim.copy_matrix_into(odd)
    assert np.array_equal(odd[:nnz], pageable[:nnz])


def test_async_system_copies_overlap_the_next_assembly(gpulib):
    """copy_system_async snapshots each assembled system before the next
    assembly overwrites it: two assemblies with different control nets,
    each copied asynchronously, equal the synchronous copies."""
    torch = pytest.importorskip("torch")
    patches, ng = W.config2(nel=6)
    sim = G.SIM(n_gauss=ng, ke_precision=G.KE_SPLIT_TF32)
    W.load_into(sim, patches)
    sim.preprocess()
    coefs = [np.ascontiguousarray(patches[0].coefs, dtype=np.float64)]
    moved = coefs[0].copy()
    moved[:, :3] *= 1.1
    coefs.append(moved)
    want = []
    for c in coefs:
        sim.update_coefs(1, c)
        sim.assembleSystem()
        want.append((sim.matrix_values(), sim.rhs()))
    nnz, neq = sim.sizes.nnz, sim.sizes.neq
    K = [torch.empty(nnz, dtype=torch.float64).pin_memory().numpy() for _ in range(2)]
    b = [torch.empty(neq, dtype=torch.float64).pin_memory().numpy() for _ in range(2)]
    for i, c in enumerate(coefs):
        sim.update_coefs(1, c)
        sim.assembleSystem(sync=False)
        sim.copy_system_async(K[i], b[i])
    sim.copy_wait()
    for i in range(2):
        assert np.array_equal(K[i], want[i][0]) and np.array_equal(b[i], want[i][1])
    assert not np.array_equal(want[0][0], want[1][0])
