"""Kronecker preconditioner and learned coarse correction, through the C ABI.

- the network's loss and gradient from the library's training kernels
  against the FP64 numpy oracle (oracle/mlp.py);
- the stored (residual, error) pairs against the oracle's restriction of
  the FP64 solution;
- flexible CG with the Kronecker preconditioner and with the learned
  correction reaching the FP64 relative residual 1e-10 on the 3D Poisson
  family with a log-normal conductivity (p = 3), with the solution equal to
  plain mixed-precision PCG's;
- the A/B comparison of what the trained network gains over the method
  without it, on a held-out seed;
- the fallback when the network returns NaN, and the weight checkpoint.
"""
import numpy as np
import pytest

from ifem_gb300 import ifemgpu as G
from ifem_gb300 import workloads as W
from oracle import mlp

pytestmark = pytest.mark.gpu

SEED0 = 4100


def poisson_model(nel=12, p=3, seed=SEED0, ke=G.KE_SPLIT_TF32):
    patches, ng = W.config4(nel=nel, p=p, seed=seed)
    sim = G.SIM(n_gauss=ng, ke_precision=ke)
    W.load_into(sim, patches)
    sim.preprocess()
    sim.assembleSystem()
    return sim, patches


def new_field(patches, seed):
    rng = np.random.default_rng(seed)
    return W.gaussian_field_3d(rng, patches[0].coefs[:, :3])


def test_training_gradients_match_oracle(gpulib):
    sim, _ = poisson_model(nel=6)
    info = sim.learn_setup(coarse_cells=2, hidden=16, capacity=8, seed=3, field_inputs=1)
    nin, nc, nh = info["inputs"], info["coarse_unknowns"], info["hidden"]
    assert nc == 27 and nin == 54
    rng = np.random.default_rng(11)
    X = rng.standard_normal((37, nin)).astype(np.float32)
    Y = rng.standard_normal((37, nc)).astype(np.float32)
    theta, _ = sim.learn_get_weights()
    theta = theta + 0.05 * rng.standard_normal(theta.size).astype(np.float32)  # non-zero biases
    sim.learn_set_weights(theta, 1.0)
    loss, grad = sim.learn_gradients(X, Y)
    ref_loss, ref_grad = mlp.loss_and_grad(theta.astype(np.float64), X, Y, nh)
    assert abs(loss - ref_loss) <= 1e-5 * ref_loss
    # FP32 sums of at most a few hundred terms: 1e-4 of the largest entry
    assert np.abs(grad - ref_grad).max() <= 1e-4 * np.abs(ref_grad).max()


def test_collected_pairs_match_oracle_restriction(gpulib):
    sim, patches = poisson_model(nel=8)
    m = 3
    sim.learn_setup(coarse_cells=m, hidden=16, capacity=64, seed=1, field_inputs=1)
    x_ref, _ = sim.solveSystem(method=G.PCG_FP64, rtol=1e-12, max_inner=20000)
    n = sim.learn_collect(xstar=x_ref, stride=4, rtol=1e-6)
    assert n >= 2
    X, Y = sim.learn_pairs()
    sam = sim.getSAM()
    pc = patches[0]
    R = mlp.restriction(pc.knots, pc.degree, pc.ncoef, sam.meqn, sam.madof, 1, m)
    b = sim.rhs()
    # the first pair is iterate 0: residual b/|b|, error x*/|b|
    rc = R @ (b / np.linalg.norm(b))
    nrm = np.linalg.norm(rc)
    Rn = R / np.maximum(R.sum(1, keepdims=True), 1e-300)
    nc = R.shape[0]
    assert np.abs(X[0, :nc] - rc / nrm).max() <= 1e-5
    ec = Rn @ (x_ref / np.linalg.norm(b)) / nrm
    assert np.abs(Y[0] - ec).max() <= 1e-4 * np.abs(ec).max()
    # field inputs: normalised trilinear average of log kappa over all control points
    g = np.asarray(pc.log_kappa)
    madof_all = np.arange(1, pc.nnod + 2, dtype=np.int32)
    meqn_all = np.arange(1, pc.nnod + 1, dtype=np.int32)
    Rf = mlp.restriction(pc.knots, pc.degree, pc.ncoef, meqn_all, madof_all, 1, m)
    f = (Rf @ g) / Rf.sum(1)
    assert np.abs(X[0, nc:] - f).max() <= 1e-5 * max(1.0, np.abs(f).max())


def test_kronecker_pcg_matches_plain_pcg(gpulib):
    sim, _ = poisson_model(nel=16)
    x0, i0 = sim.solveSystem(method=G.PCG_MIXED, rtol=1e-10)
    x1, i1 = sim.solveSystem(method=G.PCG_MIXED, rtol=1e-10, precond=G.PRECOND_KRONECKER)
    assert i0.relres <= 1e-10 and i1.relres <= 1e-10
    assert np.abs(x1 - x0).max() <= 1e-8 * np.abs(x0).max()
    print(f"\nJacobi PCG {i0.inner_iters} its {i0.device_ms:.2f} ms, "
          f"Kronecker {i1.inner_iters} its {i1.device_ms:.2f} ms")
    assert i1.inner_iters * 3 <= i0.inner_iters


def test_kronecker_elasticity(gpulib):
    patches, ng = W.config2(nel=8)
    sim = G.SIM(n_gauss=ng, ke_precision=G.KE_SPLIT_TF32)
    W.load_into(sim, patches)
    sim.preprocess()
    sim.assembleSystem()
    x0, i0 = sim.solveSystem(method=G.PCG_MIXED, rtol=1e-10)
    x1, i1 = sim.solveSystem(method=G.PCG_MIXED, rtol=1e-10, precond=G.PRECOND_KRONECKER)
    assert i1.relres <= 1e-10
    assert np.abs(x1 - x0).max() <= 1e-8 * np.abs(x0).max()
    assert i1.inner_iters < i0.inner_iters


def test_kronecker_rejects_fp64_method(gpulib):
    sim, _ = poisson_model(nel=4)
    x = np.zeros(sim.sizes.neq)
    info = G.SolveInfo()
    o = G.SolverOptions(G.PCG_FP64, 1e-10, 1, 100, 1e-4, G.PRECOND_KRONECKER)
    assert sim.lib.ifemgpu_solve(sim.ctx, G.C.byref(o), G._ptr(x), G.C.byref(info)) == G.INVALID_ARG


def train_on_seeds(sim, patches, seeds, stride=1):
    for s in seeds:
        sim.update_field(1, G.FIELD_LOG_KAPPA, new_field(patches, s))
        sim.assembleSystem()
        sim.learn_collect(stride=stride, rtol=1e-6)
    return sim.learn_train(epochs=40, batch=64, lr=1e-3, seed=5)


def test_learned_fcg_ab_on_held_out_seed(gpulib):
    sim, patches = poisson_model(nel=16)
    sim.learn_setup(coarse_cells=4, hidden=256, capacity=20000, seed=2, field_inputs=1)
    loss = train_on_seeds(sim, patches, range(SEED0 + 1, SEED0 + 13))
    train_mse = sim.learn_evaluate()
    # held-out seed
    sim.update_field(1, G.FIELD_LOG_KAPPA, new_field(patches, SEED0 + 999))
    sim.assembleSystem()
    sim.learn_clear()
    sim.learn_collect(stride=1, rtol=1e-6)
    test_mse = sim.learn_evaluate()
    xp, ip = sim.solveSystem(method=G.PCG_MIXED, rtol=1e-10)
    xk, ik = sim.solveSystem(method=G.PCG_MIXED, rtol=1e-10, precond=G.PRECOND_KRONECKER)
    xl, il = sim.solveSystem(method=G.FCG_LEARNED, rtol=1e-10, precond=G.PRECOND_KRONECKER)
    xj, ij = sim.solveSystem(method=G.FCG_LEARNED, rtol=1e-10, precond=G.PRECOND_JACOBI)
    print(f"\ntrain loss {loss:.3e} mse {train_mse:.3e}, held-out mse {test_mse:.3e}"
          f"\nplain Jacobi PCG   {ip.inner_iters:5d} its {ip.device_ms:8.2f} ms"
          f"\nKronecker FCG      {ik.inner_iters:5d} its {ik.device_ms:8.2f} ms"
          f"\nKronecker+network  {il.inner_iters:5d} its {il.device_ms:8.2f} ms fallbacks {il.fallbacks}"
          f"\nJacobi+network     {ij.inner_iters:5d} its {ij.device_ms:8.2f} ms fallbacks {ij.fallbacks}")
    for x, i in ((xk, ik), (xl, il), (xj, ij)):
        assert i.relres <= 1e-10
        assert np.abs(x - xp).max() <= 1e-8 * np.abs(xp).max()
    assert test_mse < 1.0       # better than predicting zero (targets have unit RMS)


def test_learned_fallback_on_nan_network(gpulib):
    sim, patches = poisson_model(nel=8)
    sim.learn_setup(coarse_cells=2, hidden=32, capacity=500, seed=2, field_inputs=1)
    sim.learn_collect(stride=1, rtol=1e-6)
    sim.learn_train(epochs=2, batch=32)
    theta, scale = sim.learn_get_weights()
    theta[:] = np.nan
    sim.learn_set_weights(theta, scale)
    xp, ip = sim.solveSystem(method=G.PCG_MIXED, rtol=1e-10)
    x, info = sim.solveSystem(method=G.FCG_LEARNED, rtol=1e-10, precond=G.PRECOND_KRONECKER)
    assert info.fallbacks >= 1
    assert info.relres <= 1e-10
    assert np.abs(x - xp).max() <= 1e-8 * np.abs(xp).max()


def test_weight_checkpoint_roundtrip(gpulib):
    sim, patches = poisson_model(nel=8)
    sim.learn_setup(coarse_cells=2, hidden=32, capacity=500, seed=2, field_inputs=1)
    sim.learn_collect(stride=1, rtol=1e-6)
    sim.learn_train(epochs=5, batch=32)
    theta, scale = sim.learn_get_weights()
    x1, i1 = sim.solveSystem(method=G.FCG_LEARNED, rtol=1e-10, precond=G.PRECOND_KRONECKER)
    sim.learn_setup(coarse_cells=2, hidden=32, capacity=500, seed=99, field_inputs=1)
    sim.learn_set_weights(theta, scale)
    x2, i2 = sim.solveSystem(method=G.FCG_LEARNED, rtol=1e-10, precond=G.PRECOND_KRONECKER)
    assert i1.inner_iters == i2.inner_iters
    assert np.array_equal(x1, x2)


def test_learned_solve_needs_training(gpulib):
    sim, _ = poisson_model(nel=4)
    x = np.zeros(sim.sizes.neq)
    info = G.SolveInfo()
    o = G.SolverOptions(G.FCG_LEARNED, 1e-10, 20, 1000, 1e-4, 0)
    assert sim.lib.ifemgpu_solve(sim.ctx, G.C.byref(o), G._ptr(x), G.C.byref(info)) == G.NOT_READY


def test_pairs_from_kronecker_iterates(gpulib):
    """Pairs collected along flexible CG with the Kronecker preconditioner:
    iterate 0 is the same pair as along Jacobi-PCG (x = 0), the run stops
    after far fewer iterates, and every pair is finite."""
    sim, _ = poisson_model(nel=8)
    sim.learn_setup(coarse_cells=3, hidden=16, capacity=2000, seed=1, field_inputs=1)
    n_j = sim.learn_collect(stride=1, rtol=1e-6, precond=G.PRECOND_JACOBI)
    Xj, Yj = sim.learn_pairs()
    sim.learn_clear()
    n_k = sim.learn_collect(stride=1, rtol=1e-6, precond=G.PRECOND_KRONECKER)
    Xk, Yk = sim.learn_pairs()
    assert 2 <= n_k < n_j
    assert np.abs(Xk[0] - Xj[0]).max() <= 1e-6 and np.abs(Yk[0] - Yj[0]).max() <= 1e-6
    assert np.isfinite(Xk).all() and np.isfinite(Yk).all()


def csc_matrix(sim):
    import scipy.sparse as sp
    sam = sim.getSAM()
    n = sim.sizes.neq
    return sp.csc_matrix((sim.matrix_values(), sam.rowidx, sam.colptr), shape=(n, n))


def test_complement_pairs_of_the_kronecker_step(gpulib):
    """Complement pairs along flexible CG with the Kronecker preconditioner:
    the first pair (x = 0, r0 = b/|b|, z0 = M r0) has the input
    R (r0 - A z0) / |R (r0 - A z0)| and the target
    Rn (x*/|b| - z0) / |R (r0 - A z0)|."""
    sim, patches = poisson_model(nel=8)
    m = 3
    sim.learn_setup(coarse_cells=m, hidden=16, capacity=64, seed=1, field_inputs=0)
    x_ref, _ = sim.solveSystem(method=G.PCG_FP64, rtol=1e-12, max_inner=20000)
    sim.learn_collect(xstar=x_ref, stride=4, rtol=1e-6, precond=G.PRECOND_KRONECKER)
    sim.learn_set_target(G.LEARN_TARGET_COMPLEMENT)
    assert sim.learn_info()["pairs"] == 0          # changing the mode forgets the pairs
    sim.learn_collect(xstar=x_ref, stride=4, rtol=1e-6, precond=G.PRECOND_KRONECKER)
    Xc, Yc = sim.learn_pairs()
    sam = sim.getSAM()
    pc = patches[0]
    R = mlp.restriction(pc.knots, pc.degree, pc.ncoef, sam.meqn, sam.madof, 1, m)
    Rn = R / np.maximum(R.sum(1, keepdims=True), 1e-300)
    A = csc_matrix(sim)
    b = sim.rhs()
    r0 = b / np.linalg.norm(b)
    z0 = sim.apply_preconditioner(r0, G.PRECOND_KRONECKER)
    rc1 = R @ (r0 - A @ z0)
    nrm = np.linalg.norm(rc1)
    assert np.abs(Xc[0] - rc1 / nrm).max() <= 1e-4
    want = Rn @ (x_ref / np.linalg.norm(b) - z0) / nrm
    assert np.abs(Yc[0] - want).max() <= 1e-3 * np.abs(want).max()
    with pytest.raises(G.IfemGpuError):
        sim.learn_set_target(7)


@pytest.mark.parametrize("kind", ["poisson", "elasticity"])
def test_galerkin_coarse_matrix(gpulib, kind):
    """The learned step's Galerkin coarse matrix R A R^T against numpy's
    product of the FP64 matrix with the oracle's restriction (FP32 sums:
    1e-5 of the largest entry)."""
    if kind == "poisson":
        sim, patches = poisson_model(nel=8)
        npv = 1
    else:
        patches, ng = W.config2(nel=8)
        sim = G.SIM(n_gauss=ng, ke_precision=G.KE_SPLIT_TF32)
        W.load_into(sim, patches)
        sim.preprocess()
        sim.assembleSystem()
        npv = 3
    m = 2
    sim.learn_setup(coarse_cells=m, hidden=16, capacity=8, seed=1, field_inputs=0)
    Ac = sim.learn_coarse_matrix()
    sam = sim.getSAM()
    pc = patches[0]
    R = mlp.restriction(pc.knots, pc.degree, pc.ncoef, sam.meqn, sam.madof, npv, m)
    ref = (R @ (csc_matrix(sim) @ R.T))
    assert Ac.shape == ref.shape
    assert np.abs(Ac - ref).max() <= 1e-5 * np.abs(ref).max()


def test_untrained_network_costs_no_convergence(gpulib):
    """The energy-optimal coefficient: a network with its initial random
    weights still reaches the FP64 residual with about the Kronecker
    iteration count (the step along a useless direction is near zero)."""
    sim, _ = poisson_model(nel=16)
    sim.learn_setup(coarse_cells=4, hidden=64, capacity=8, seed=3, field_inputs=1)
    theta, scale = sim.learn_get_weights()
    sim.learn_set_weights(theta, scale)                # marks the network usable
    xk, ik = sim.solveSystem(method=G.PCG_MIXED, rtol=1e-10, precond=G.PRECOND_KRONECKER)
    xl, il = sim.solveSystem(method=G.FCG_LEARNED, rtol=1e-10, precond=G.PRECOND_KRONECKER)
    print(f"\nKronecker FCG {ik.inner_iters} its, with an untrained network {il.inner_iters} its")
    assert il.relres <= 1e-10 and il.fallbacks == 0
    assert il.inner_iters <= 1.25 * ik.inner_iters + 4
    assert np.abs(xl - xk).max() <= 1e-8 * np.abs(xk).max()


def test_learned_rejects_coarse_cells_narrower_than_coupling(gpulib):
    sim, _ = poisson_model(nel=8)
    sim.learn_setup(coarse_cells=4, hidden=16, capacity=8, seed=1, field_inputs=0)
    theta, scale = sim.learn_get_weights()
    sim.learn_set_weights(theta, scale)
    x = np.zeros(sim.sizes.neq)
    info = G.SolveInfo()
    o = G.SolverOptions(G.FCG_LEARNED, 1e-10, 20, 1000, 1e-4, G.PRECOND_KRONECKER)
    assert sim.lib.ifemgpu_solve(sim.ctx, G.C.byref(o), G._ptr(x), G.C.byref(info)) == G.UNSUPPORTED


def bf16(a):
    """Round to BF16 (nearest even), returned as float64."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


@pytest.mark.parametrize("hidden", [160, 256])
def test_tensor_core_inference_matches_bf16_reference(gpulib, hidden):
    """The solve's inference path (BF16 tcgen05 products, FP32 accumulation in
    tensor memory, weights and each layer's inputs in BF16) against an FP64
    evaluation of the same rounded operands: 2e-3 of the largest output (FP32
    sums of up to a few hundred products).  hidden = 160 pads the row and K
    tiles; several K tiles are summed by the last CTA of a row tile."""
    sim, _ = poisson_model(nel=8)
    info = sim.learn_setup(coarse_cells=2, hidden=hidden, capacity=4, seed=4, field_inputs=1)
    nc, nin, nh = info["coarse_unknowns"], info["inputs"], info["hidden"]
    theta, scale = sim.learn_get_weights()
    rng = np.random.default_rng(17)
    theta = theta + 0.05 * rng.standard_normal(theta.size).astype(np.float32)
    sim.learn_set_weights(theta, scale)
    sim.learn_collect(stride=1, rtol=1e-2)
    X, _ = sim.learn_pairs(0, 1)
    feat = X[0, nc:].astype(np.float64)
    rc = rng.standard_normal(nc).astype(np.float32)
    y = sim.learn_forward(rc)
    W1, b1, W2, b2, W3, b3 = mlp.unpack(theta, nin, nh, nc)
    x0 = np.concatenate([rc.astype(np.float64) / np.linalg.norm(rc.astype(np.float64)), feat])
    h1 = np.maximum(bf16(W1) @ bf16(x0) + b1, 0.0)
    h2 = np.maximum(bf16(W2) @ bf16(h1) + b2, 0.0)
    ref = bf16(W3) @ bf16(h2) + b3
    assert np.isfinite(y).all()
    assert np.abs(y - ref).max() <= 2e-3 * np.abs(ref).max()
