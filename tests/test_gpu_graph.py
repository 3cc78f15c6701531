"""The captured assemble -> solve step (ifemgpu_graph_capture / _launch): one
CUDA graph holding the assembly, the solver prologue and the device-driven
refinement and inner loops (conditional WHILE nodes).  A replay must give
bitwise the K, b and x of ifemgpu_assemble + ifemgpu_solve with the same
options -- after the model's field or control net changed, too."""
import numpy as np
import pytest

from ifem_gb300 import ifemgpu as G
from ifem_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def model(patches, ng):
    sim = G.SIM(n_gauss=ng, ke_precision=G.KE_SPLIT_TF32)
    W.load_into(sim, patches)
    sim.preprocess()
    return sim


@pytest.mark.parametrize("precond", [G.PRECOND_JACOBI, G.PRECOND_KRONECKER])
def test_graph_step_equals_uncaptured_calls(gpulib, precond):
    patches, ng = W.config4(nel=12, grid=16)
    pts = patches[0].coefs[:, :3]
    fields = [patches[0].log_kappa] + [
        W.gaussian_field_3d(np.random.default_rng(900 + k), pts, grid=16) for k in range(2)]
    ref = model(patches, ng)
    cap = model(patches, ng)
    opts = dict(rtol=1e-10, inner_rtol=1e-4, precond=precond)
    cap.graph_capture(**opts)
    for f in fields:
        ref.update_field(1, G.FIELD_LOG_KAPPA, f)
        ref.assembleSystem()
        x0, i0 = ref.solveSystem(**opts)
        cap.update_field(1, G.FIELD_LOG_KAPPA, f)
        x1, i1 = cap.graph_launch()
        assert np.array_equal(cap.matrix_values(), ref.matrix_values())
        assert np.array_equal(cap.rhs(), ref.rhs())
        assert np.array_equal(x1, x0)
        assert (i1.outer_iters, i1.inner_iters) == (i0.outer_iters, i0.inner_iters)
        assert i1.relres == i0.relres and i1.relres <= 1e-10


def test_graph_step_elasticity_new_control_net(gpulib):
    patches, ng = W.config2(nel=6)
    ref = model(patches, ng)
    cap = model(patches, ng)
    cap.graph_capture(rtol=1e-10)
    coefs = np.ascontiguousarray(patches[0].coefs, dtype=np.float64)
    for scale in (1.0, 1.05):
        c = coefs.copy()
        c[:, :3] *= scale
        ref.update_coefs(1, c)
        ref.assembleSystem()
        x0, i0 = ref.solveSystem(rtol=1e-10)
        cap.update_coefs(1, c)
        x1, i1 = cap.graph_launch()
        assert np.array_equal(cap.matrix_values(), ref.matrix_values())
        assert np.array_equal(x1, x0) and i1.inner_iters == i0.inner_iters


def test_graph_step_rejects_other_methods(gpulib):
    patches, ng = W.config2(nel=3)
    sim = model(patches, ng)
    o = G.SolverOptions(G.PCG_FP64, 1e-10, 20, 1000, 1e-4, G.PRECOND_JACOBI)
    assert sim.lib.ifemgpu_graph_capture(sim.ctx, o) == G.UNSUPPORTED
    x, info = sim.graph_launch(check=False)
    assert sim.lib.ifemgpu_graph_launch(sim.ctx, None, None) == G.NOT_READY
