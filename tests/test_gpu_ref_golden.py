"""GPU assembly against global systems assembled by IFEM's own code
(tests/golden/ref_systems.npz, see tests/golden/make_ref_systems.py), through
the C ABI.

FP64 element arithmetic: pattern, MADOF and MEQN bit-exact, K and b within
1e-12 of max|K|.  Split precision (3xTF32 tensor cores where the patch is p=2
elasticity, FP32 CUDA cores otherwise): within 5e-6 of max|K|.
"""
import os

import numpy as np
import pytest

from ifem_gb300 import ifemgpu as G
from ifem_gb300 import workloads as W

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "ref_systems.npz")


def _cases():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_ref_systems", os.path.join(HERE, "golden", "make_ref_systems.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.cases()


CASES = _cases()


def golden(name):
    z = np.load(FIX)
    return {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(name + "/")}


@pytest.mark.parametrize("ke,tol", [(G.KE_FP64, 1e-12), (G.KE_SPLIT_TF32, 5e-6)],
                         ids=["fp64", "split"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_matches_reference_system(gpulib, name, ke, tol):
    patches, ng = CASES[name][:2]
    conns = CASES[name][2] if len(CASES[name]) > 2 else ()
    ref = golden(name)
    sim = G.SIM(n_gauss=ng, ke_precision=ke)
    W.load_into(sim, patches, conns)
    sim.preprocess()
    sim.assembleSystem()
    sam = sim.getSAM()
    np.testing.assert_array_equal(sam.madof, ref["madof"])
    np.testing.assert_array_equal(sam.meqn, ref["meqn"])
    np.testing.assert_array_equal(sam.colptr, ref["IA"])
    np.testing.assert_array_equal(sam.rowidx, ref["JA"])
    K = sim.matrix_values()
    assert np.abs(K - ref["A"]).max() <= tol * np.abs(ref["A"]).max()
    if "b" in ref:
        b = sim.rhs()
        assert np.abs(b - ref["b"]).max() <= tol * np.abs(ref["b"]).max()


def test_gpu_dump_round_trip(gpulib, tmp_path):
    """ifemgpu_dump_system of a GPU assembly reads back to the same values
    (17 significant digits) and pattern, in IFEM's MatrixMarket layout."""
    patches, ng = CASES["c1_poisson2d_p2"][:2]
    sim = G.SIM(n_gauss=ng, ke_precision=G.KE_FP64)
    W.load_into(sim, patches)
    sim.preprocess()
    sim.assembleSystem()
    sim.dump_system(tmp_path / "A.mtx", tmp_path / "b.mtx", G.DUMP_MATRIX_MARKET)
    lines = (tmp_path / "A.mtx").read_text().splitlines()
    assert lines[0].startswith("%%MatrixMarket matrix coordinate real general")
    n, _, nnz = (int(v) for v in lines[2].split())
    ent = np.array([[float(v) for v in ln.split()] for ln in lines[3:3 + nnz]])
    sam = sim.getSAM()
    cols = np.repeat(np.arange(n), np.diff(sam.colptr)) + 1
    np.testing.assert_array_equal(ent[:, 0], sam.rowidx + 1)
    np.testing.assert_array_equal(ent[:, 1], cols)
    np.testing.assert_array_equal(ent[:, 2], sim.matrix_values())
    b = np.array([float(v) for v in (tmp_path / "b.mtx").read_text().split()[7:]])
    np.testing.assert_array_equal(b, sim.rhs())


SEC = sorted(n for n in CASES if "sec" in golden(n))


@pytest.mark.parametrize("ke,tol", [(G.KE_FP64, 1e-10), (G.KE_SPLIT_TF32, 2e-5)],
                         ids=["fp64", "split"])
@pytest.mark.parametrize("name", SEC)
def test_gpu_secondary_matches_reference(gpulib, name, ke, tol):
    """Gauss-point flux (Poisson) / stress (elasticity) of a seeded DOF vector
    against the values evaluated with IFEM's own utl::Jacobian (fixture key
    "sec"): FP64 mode to 1e-10, split mode (FP32 point arithmetic) to 2e-5 of
    the largest value."""
    patches, ng = CASES[name][:2]
    ref = golden(name)
    sim = G.SIM(n_gauss=ng, ke_precision=ke)
    W.load_into(sim, patches)
    sim.preprocess()
    sim.assembleSystem()
    nel, nq, ncomp = ref["sec"].shape
    sec = sim.secondary_solution(1, ref["u"], nq, ncomp)
    assert np.abs(sec - ref["sec"]).max() <= tol * np.abs(ref["sec"]).max()