"""System dumps in IFEM's text formats (SparseMatrix::dump, StdVector::dump
as SIMbase::dumpEqSys writes them), byte for byte against files IFEM's own
code wrote for the golden system c0_poisson2d_small
(tests/golden/ref_dump/, tests/golden/make_ref_systems.py).  The writer is a
host function of libifemgpu.so and needs no GPU."""
import os

import numpy as np
import pytest

from ifem_gb300 import ifemgpu as G

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "ref_systems.npz")
DUMPS = os.path.join(HERE, "golden", "ref_dump")


@pytest.fixture(scope="module")
def lib():
    from ifem_gb300 import build
    build.ensure_built()
    return G.load_library()


@pytest.mark.parametrize("fmt,ext", [(G.DUMP_FLAT, "flat"), (G.DUMP_MATLAB, "m"),
                                     (G.DUMP_MATRIX_MARKET, "mtx")])
def test_writer_matches_ifem_dump(lib, tmp_path, fmt, ext):
    z = np.load(FIX)
    g = {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith("c0_poisson2d_small/")}
    mat, rhs = tmp_path / f"A.{ext}", tmp_path / f"b.{ext}"
    G.write_system(g["IA"], g["JA"], g["A"], g["b"], mat, rhs, fmt, 1e-12, lib=lib)
    for got, ref in ((mat, f"A.{ext}"), (rhs, f"b.{ext}")):
        assert got.read_bytes() == open(os.path.join(DUMPS, ref), "rb").read(), ref


def test_writer_rejects_bad_format(lib, tmp_path):
    with pytest.raises(G.IfemGpuError):
        G.write_system([0, 1], [0], [1.0], [1.0], tmp_path / "A", None, 7, 0.0, lib=lib)
