"""C-ABI library on the CPU: exported symbols, and the host-side model logic
(topology, SAM numbering, compressed-column pattern) of a host-only context
(device = -1) against the oracle and IFEM's golden vectors.  No GPU work."""
import ctypes as C
import json
import os
import re

import numpy as np
import pytest

from ifem_gb300 import ifemgpu as G
from ifem_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def header_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            with open(os.path.join(ROOT, "include", name)) as f:
                txt = f.read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            syms |= set(re.findall(r"\b(ifemgpu_\w+)\s*\(", txt))
    return syms


def test_library_exports_every_declared_symbol(gpulib):
    syms = header_symbols()
    assert syms, "no declarations found"
    for s in sorted(syms):
        assert hasattr(gpulib, s), f"{s} declared in include/ but not exported"
    assert set(G.EXPORTS) <= syms
    assert gpulib.ifemgpu_abi_version() == 2


def host_sim(n_gauss=4):
    return G.SIM(n_gauss=n_gauss, device=-1)


def both(patches, ng):
    import oracle
    sim = host_sim(ng)
    W.load_into(sim, patches)
    sim.preprocess()
    orc = oracle.OracleModel(ng)
    W.load_into(orc, patches)
    orc.preprocess()
    return sim, orc


CASES = {
    "cfg1": lambda: W.config1(),
    "cfg2_small": lambda: W.config2(nel=6),
    "cfg2_p3": lambda: W.config2(nel=4, p=3),
    "cfg4_small": lambda: W.config4(nel=6, grid=16),
    "cfg3_small": lambda: W.config3(npatch=5, nmin=2, nmax=4),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_numbering_and_pattern_bit_exact(oracle_lib, name):
    patches, ng = CASES[name]()
    sim, orc = both(patches, ng)
    s = sim.sizes
    assert (s.nnod, s.nel, s.ndof, s.neq, s.nceq, s.nnz) == tuple(
        orc.sizes[k] for k in ("nnod", "nel", "ndof", "neq", "nceq", "nnz"))
    sam = sim.getSAM()
    madof, meqn = orc.sam()
    np.testing.assert_array_equal(sam.madof, madof)
    np.testing.assert_array_equal(sam.meqn, meqn)
    IA, JA = orc.pattern()
    np.testing.assert_array_equal(sam.colptr, IA)
    np.testing.assert_array_equal(sam.rowidx, JA)
    for pid, pc in enumerate(patches, 1):
        nen = int(np.prod([p + 1 for p in pc.degree]))
        np.testing.assert_array_equal(sim.mnpc(pid), orc.mnpc(pid, pc.nel, nen))


def test_zero_span_elements_and_general_coupling(oracle_lib):
    """A repeated interior knot gives zero-volume elements (skipped, IFEM
    ASMs3D.C:487-509) and a pattern that is not the index box."""
    pc = W.box_patch(2, 2, 4)
    k = np.array([0, 0, 0, 0.25, 0.5, 0.5, 1, 1, 1])   # repeated 0.5
    pc.knots[0] = k
    pc.ncoef = (len(k) - 3, pc.ncoef[1])
    g0 = W.greville(k, 2)
    g1 = W.greville(pc.knots[1], 2)
    X, Y = np.meshgrid(g0, g1, indexing="xy")
    pc.coefs = np.stack([X.ravel(), Y.ravel()], axis=1)
    pc.dirichlet = [(1, 1, 0.0)]
    sim, orc = both([pc], 3)
    assert sim.sizes.nel == orc.sizes["nel"] < (len(k) - 3 - 2) * 4
    sam = sim.getSAM()
    IA, JA = orc.pattern()
    np.testing.assert_array_equal(sam.colptr, IA)
    np.testing.assert_array_equal(sam.rowidx, JA)


@pytest.mark.parametrize("case,dirichlet", [("sam_2D_singlebasis_1P", False),
                                            ("sam_2D_singlebasis_dir_1P", True)])
def test_sam_golden_through_the_library(case, dirichlet, gpulib):
    with open(os.path.join(GOLD, "sam_refs.json")) as f:
        g = json.load(f)["cases"][case]
    sim = host_sim(2)
    pid = sim.add_patch(W.box_patch(2, 1, 2))
    sim.set_material(pid, G.POISSON)
    if dirichlet:
        sim.constrain_face(pid, 2, 1, 1.0)
    sim.preprocess()
    sam = sim.getSAM()
    assert sam.getDofCouplings() == g["couplings"]
    for node, eq in g.get("equations", {}).get("node_eq", []):
        assert sam.getEquation(node, 1) == eq


def square2(dirichlet):
    """src/LinAlg/Test/refdata/square2.g2: two bilinear one-element patches."""
    p1 = W.box_patch(2, 1, 1, size=(0.5, 1.0))
    p2 = W.box_patch(2, 1, 1, origin=(0.5, 0.0, 0.0), size=(0.5, 1.0))
    for p in (p1, p2):
        p.kind = G.POISSON
    if dirichlet:
        p2.dirichlet = [(2, 1, 1.0)]
    return [p1, p2]


@pytest.mark.parametrize("case,dirichlet", [("sam_2D_singlebasis_2P", False),
                                            ("sam_2D_singlebasis_dir_2P", True)])
def test_two_patch_sam_golden_through_the_library(case, dirichlet, gpulib):
    with open(os.path.join(GOLD, "sam_refs.json")) as f:
        g = json.load(f)["cases"][case]
    sim = host_sim(2)
    W.load_into(sim, square2(dirichlet), [tuple(g["connection"])])
    sim.preprocess()
    sam = sim.getSAM()
    assert sam.getDofCouplings() == g["couplings"]
    eqs = g.get("equations", {}).get("node_eq", [[n, n] for n in range(1, 7)])
    for node, eq in eqs:
        assert sam.getEquation(node, 1) == eq


def test_connection_errors(gpulib):
    sim = host_sim(2)
    p1, p2 = square2(False)
    W.load_into(sim, [p1, p2])
    with pytest.raises(G.IfemGpuError):
        sim.connect(1, 2, 1, 1, 0)                # a patch with itself
    with pytest.raises(G.IfemGpuError):
        sim.connect(1, 5, 2, 1, 0)                # no edge 5 in 2D
    sim.connect(1, 1, 2, 1, 0)                    # edges that do not coincide
    with pytest.raises(G.IfemGpuError):
        sim.preprocess()


def test_element_nodes_golden_through_the_library(gpulib):
    with open(os.path.join(GOLD, "elm_nodes.json")) as f:
        g = json.load(f)
    for key, p in (("linear", 1), ("quadratic", 2)):
        sim = host_sim(2)
        pid = sim.add_patch(W.box_patch(3, p, 2))
        sim.set_material(pid, G.POISSON)
        sim.preprocess()
        np.testing.assert_array_equal(sim.mnpc(pid), np.array(g[key]))


def test_errors_are_reported_not_fallen_back(gpulib):
    sim = host_sim()
    with pytest.raises(G.IfemGpuError) as e:
        sim.preprocess()                       # no patches
    assert e.value.status == G.NOT_READY
    pid = sim.add_patch(W.box_patch(3, 2, 2))
    with pytest.raises(G.IfemGpuError):
        sim.preprocess()                       # no material
    with pytest.raises(G.IfemGpuError) as e:
        sim.set_material(pid, 7)
    assert e.value.status == G.INVALID_ARG
    sim.set_material(pid, G.ELASTICITY)
    with pytest.raises(G.IfemGpuError):
        sim.constrain_face(pid, 9, 123)
    sim.preprocess()
    with pytest.raises(G.IfemGpuError) as e:
        sim.assembleSystem()                   # host-only context has no device
    assert e.value.status == G.NOT_READY
    pc2 = W.box_patch(2, 2, 2)
    sim2 = host_sim()
    pid2 = sim2.add_patch(pc2)
    with pytest.raises(G.IfemGpuError) as e:
        sim2.set_material(pid2, G.ELASTICITY)  # 2D elasticity is not implemented
    assert e.value.status == G.UNSUPPORTED
    bad = W.box_patch(3, 5, 1)                 # degree above 4
    with pytest.raises(G.IfemGpuError) as e:
        host_sim().add_patch(bad)
    assert e.value.status == G.UNSUPPORTED


FAST_CASES = dict(CASES, connected=lambda: W.connected_boxes(kind=2, nel=3, npatch=3,
                                                                rotated=True))


@pytest.mark.parametrize("name", sorted(FAST_CASES))
def test_oracle_parallel_pattern_equals_set_couplings(oracle_lib, name):
    """The oracle's parallel pattern construction (used for the large models of
    the benchmark) gives the arrays of IFEM's std::set couplings."""
    import oracle
    made = FAST_CASES[name]()
    patches, ng = made[0], made[1]
    conns = made[2] if len(made) > 2 else ()
    pats = []
    for mode in (0, 1):
        orc = oracle.OracleModel(ng)
        W.load_into(orc, patches, conns)
        orc.preprocess(pattern=mode)
        pats.append(orc.pattern())
    np.testing.assert_array_equal(pats[0][0], pats[1][0])
    np.testing.assert_array_equal(pats[0][1], pats[1][1])


@pytest.mark.parametrize("name", ["cfg2_p3", "cfg4_small", "cfg3_small"])
def test_oracle_binary_search_scatter_equals_linear(oracle_lib, name):
    """The oracle's binary-search entry lookup (used by the large parity tests)
    gives bitwise the sums of IFEM's linear std::find lookup."""
    import oracle
    patches, ng = CASES[name]()
    out = []
    for bis in (False, True):
        orc = oracle.OracleModel(ng)
        W.load_into(orc, patches)
        orc.preprocess()
        orc.set_bisect(bis)
        orc.assemble(4)
        out.append(orc.system())
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
