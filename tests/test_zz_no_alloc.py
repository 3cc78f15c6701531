"""The allocation-free solve entry point (ifemgpu_solve_noalloc).

Some callers cannot allocate device memory when they solve: an application
that gives its whole device memory to its own pool, a Newton or time-step
loop that must not synchronise on cudaMalloc, a host framework that owns the
allocator.  ifemgpu_solve_noalloc serves them with a fixed workspace inside
the library.  Here it is called through the C ABI and checked against the
allocating ifemgpu_solve (FP64 Jacobi-PCG, same tolerance and cap) on two
calls in a row: the solutions must agree to 1e-12 relative (they run the
same kernels, so they are expected to be identical).  This file is collected
last so that a run stopping at the first failure has run every other test.
"""
import numpy as np
import pytest

from ifem_gb300 import ifemgpu as G
from ifem_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-12


def model(ke=G.KE_FP64, nel=8):
    patches, ng = W.config2(nel=nel)
    sim = G.SIM(n_gauss=ng, ke_precision=ke)
    W.load_into(sim, patches)
    sim.preprocess()
    sim.assembleSystem()
    return sim


@pytest.mark.parametrize("ke", [G.KE_FP64, G.KE_SPLIT_TF32])
def test_noalloc_solve_matches_allocating_solve(gpulib, ke):
    sim = model(ke)
    assert sim.sizes.neq <= 65536
    ref, rinfo = sim.solveSystem(method=G.PCG_FP64, rtol=1e-10, max_inner=20000)
    for _ in range(2):   # the shared workspace keeps the previous call's contents
        x, info, st = sim.solve_noalloc(rtol=1e-10, max_iter=20000)
        assert st == G.OK
        assert info.relres <= 1e-10
        assert info.inner_iters == rinfo.inner_iters
        assert np.abs(x - ref).max() <= TOL * np.abs(ref).max()


def test_noalloc_first_solve_allocates_no_device_memory(gpulib):
    """On a freshly assembled model the first solve is the allocation-free one:
    the device's free memory is the same before and after it (the context has
    no solver workspace yet, so an allocation would show), and its solution
    equals the allocating solve's."""
    torch = pytest.importorskip("torch")
    warm = model(G.KE_FP64, nel=4)           # loads the solver kernels once
    warm.solve_noalloc(rtol=1e-10, max_iter=20000)
    sim = model(G.KE_FP64)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    x, info, st = sim.solve_noalloc(rtol=1e-10, max_iter=20000)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert st == G.OK and info.relres <= 1e-10
    assert free1 == free0, (free0, free1)
    ref, rinfo = sim.solveSystem(method=G.PCG_FP64, rtol=1e-10, max_inner=20000)
    assert info.inner_iters == rinfo.inner_iters
    assert np.abs(x - ref).max() <= TOL * np.abs(ref).max()


def test_noalloc_rejects_systems_above_its_limit(gpulib):
    sim = model(G.KE_SPLIT_TF32, nel=20)     # 3 * 22 * 22 * 21 = 30,492 equations: fits
    assert sim.sizes.neq <= 65536
    big = model(G.KE_SPLIT_TF32, nel=28)     # 3 * 30 * 30 * 29 = 78,300 equations
    assert big.sizes.neq > 65536
    x, info, st = big.solve_noalloc(check=False)
    assert st == G.INVALID_ARG
    assert b"65536" in big.lib.ifemgpu_last_error(big.ctx)
