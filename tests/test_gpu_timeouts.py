"""The failure path of the bounded device waits, made to run out on purpose
without faulting the GPU (ifemgpu_debug_waits): one element's done flag is
never published, or its control-point copy never issued, and the limits are
short.  The kernels must return, the host must report IFEMGPU_DEVICE_TIMEOUT
and refuse to hand out or solve the invalid system, and after the hooks are
cleared the next assembly must be exact again."""
import numpy as np
import pytest

from ifem_gb300 import ifemgpu as G
from ifem_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def sim_of(patches, ng, ke, colour_passes=0):
    sim = G.SIM(n_gauss=ng, ke_precision=ke, colour_passes=colour_passes)
    W.load_into(sim, patches)
    sim.preprocess()
    return sim


def run_withheld(sim, ref, flag_spin, copy_spin, element):
    L, c = sim.lib, sim.ctx
    assert L.ifemgpu_debug_waits(c, flag_spin, copy_spin, 1, element) == G.OK
    assert L.ifemgpu_assemble(c, 1) == G.DEVICE_TIMEOUT
    assert b"bounded device wait" in L.ifemgpu_last_error(c)
    # the system is marked invalid: no copies, no solve
    K = np.zeros(sim.sizes.nnz)
    assert L.ifemgpu_copy_matrix(c, G._ptr(K)) == G.NOT_READY
    x, info = sim.solveSystem(check=False)
    assert L.ifemgpu_solve(c, G.SolverOptions(G.PCG_MIXED, 1e-10, 20, 1000, 1e-4, 0),
                           G._ptr(x), info) == G.NOT_READY
    # hooks cleared: the next assembly is the reference again, bit for bit
    assert L.ifemgpu_debug_waits(c, 0, 0, 0, 0) == G.OK
    assert L.ifemgpu_assemble(c, 1) == G.OK
    assert np.array_equal(sim.matrix_values(), ref.matrix_values())
    assert np.array_equal(sim.rhs(), ref.rhs())


def test_flag_wait_of_persistent_generic_pass_times_out(gpulib):
    patches, ng = W.config2(nel=4)
    ref = sim_of(patches, ng, G.KE_FP64, colour_passes=2)
    ref.assembleSystem()
    sim = sim_of(patches, ng, G.KE_FP64, colour_passes=2)
    run_withheld(sim, ref, flag_spin=256, copy_spin=0, element=0)


@pytest.mark.parametrize("which", ["elasticity", "poisson"])
def test_copy_wait_of_tensor_core_kernel_times_out(gpulib, which):
    patches, ng = W.config2(nel=4) if which == "elasticity" else W.config4(nel=4, grid=16)
    ref = sim_of(patches, ng, G.KE_SPLIT_TF32)
    ref.assembleSystem()
    sim = sim_of(patches, ng, G.KE_SPLIT_TF32)
    sim.assembleSystem()                    # tuned and captured once with the default limits
    run_withheld(sim, ref, flag_spin=0, copy_spin=64, element=5)
