"""The CPU oracle against the golden vectors of IFEM's own unit tests
(fixtures in tests/golden/, extracted by tests/golden/make_golden.py)."""
import json
import os

import numpy as np
import pytest

from ifem_gb300 import workloads as W

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def gold(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


def unit_patch(dim, p, nel):
    """Identity-map patch on the unit square/cube (IFEM's default geometry,
    refined and order-elevated)."""
    return W.box_patch(dim, p, nel)


def test_gauss_rules_match_ifem_tables(oracle_lib):
    # GaussQuadrature.C tabulates 1..10 point rules: 1..9 points to ~1 ulp
    # of the exact rule, the 10-point rule to 8 decimal digits only.
    g = gold("gauss_tables.json")
    for n in range(1, 11):
        x, w = oracle_lib.gauss(n)
        ref = g["rules"][str(n)]
        tol = 1e-8 if n == 10 else 5e-16
        np.testing.assert_allclose(x, ref["xi"], rtol=0, atol=tol)
        np.testing.assert_allclose(w, ref["w"], rtol=0, atol=tol)


@pytest.mark.parametrize("n", range(1, 11))
def test_gauss_integrates_polynomials(oracle_lib, n):
    # TestGaussQuadrature.Integrate: sum_p int x^p over [-1,1]
    x, w = oracle_lib.gauss(n)
    res = sum(w[i] * x[i] ** p for i in range(n) for p in range(n))
    exa = sum((1 - (-1) ** (p + 1)) / (p + 1) for p in range(n))
    assert abs(res - exa) <= (1e-7 if n == 10 else 1e-14) * abs(exa)


def test_laplacian_and_stress_operators(oracle_lib):
    g = gold("equal_order_operators.json")
    dNdX = np.array(g["dNdX"])
    # EqualOrderOperators::Weak::Laplacian, scalar block
    eK = oracle_lib.op_laplacian(dNdX)
    np.testing.assert_allclose(eK.ravel(), g["laplacian_scalar"], rtol=1e-15)
    # stress formulation (lambda = 0, mu = 1 of the elasticity operator)
    eK = oracle_lib.op_elasticity(dNdX, 0.0, 1.0)
    np.testing.assert_allclose(eK.ravel(), g["laplacian_stress"], rtol=1e-15)
    # component interleaving EM(nf*(i-1)+k, nf*(j-1)+k) of the multi-block form
    A = np.array(g["laplacian_scalar"]).reshape(2, 2)
    np.testing.assert_allclose(np.kron(A, np.eye(2)).ravel(), g["laplacian_multi"])


def test_jacobian3d_on_refined_trilinear_cube(oracle_lib):
    g = gold("jacobian3d.json")
    pc = unit_patch(3, 1, g["refine"] + 1)
    m = oracle_lib.OracleModel(2)
    pid = m.add_patch(pc)
    m.set_material(pid, 1)
    m.preprocess()
    N, dNdu, nodes = basis(oracle_lib, m, pid, g["param"], 8, 3)
    # element 2 (1-based): the second element along u
    mnpc = m.mnpc(pid, pc.nel, 8)
    Xn = pc.coefs[mnpc[g["element"] - 1]]
    det, J, dNdX = oracle_lib.jacobian(3, Xn, dNdu)
    assert det == pytest.approx(g["det"], rel=1e-14)
    np.testing.assert_allclose(J, np.eye(3), atol=1e-14)
    np.testing.assert_allclose(dNdX.T.ravel(), g["dNdX_column_major"], atol=1e-13)


def basis(oracle_lib, m, pid, u, nen, dim):
    import ctypes as C
    uu = np.array(u, dtype=np.float64)
    N = np.zeros(nen)
    dN = np.zeros(nen * dim)
    nodes = np.zeros(nen, dtype=np.int32)
    oracle_lib.lib().ifo_basis(m.h, pid, uu.ctypes.data_as(C.c_void_p),
                               N.ctypes.data_as(C.c_void_p), dN.ctypes.data_as(C.c_void_p),
                               nodes.ctypes.data_as(C.c_void_p))
    return N, dN.reshape(dim, nen).T, nodes


def test_bilinear_surface_basis(oracle_lib):
    g = gold("spline_surface.json")
    pc = unit_patch(2, 1, 1)
    m = oracle_lib.OracleModel(2)
    pid = m.add_patch(pc)
    m.set_material(pid, 1)
    m.preprocess()
    N, dNdu, _ = basis(oracle_lib, m, pid, g["param"], 4, 2)
    np.testing.assert_allclose(N, g["N"], rtol=1e-14)
    np.testing.assert_allclose(dNdu, g["dNdU"], rtol=1e-14)


@pytest.mark.parametrize("key,p", [("linear", 1), ("quadratic", 2)])
def test_element_nodes_of_refined_cube(oracle_lib, key, p):
    g = gold("elm_nodes.json")
    pc = unit_patch(3, p, 2)
    m = oracle_lib.OracleModel(2)
    pid = m.add_patch(pc)
    m.set_material(pid, 1)
    m.preprocess()
    nen = (p + 1) ** 3
    np.testing.assert_array_equal(m.mnpc(pid, 8, nen), np.array(g[key]))


def sam_model(lib_factory, dirichlet):
    pc = unit_patch(2, 1, 2)   # bilinear unit square, one knot inserted per direction
    m = lib_factory()
    pid = m.add_patch(pc)
    m.set_material(pid, 1)
    if dirichlet:
        m.constrain_face(pid, 2, 1, 1.0)   # edge 2 (+u), constant value 1.0
    m.preprocess()
    return m


@pytest.mark.parametrize("case,dirichlet", [("sam_2D_singlebasis_1P", False),
                                            ("sam_2D_singlebasis_dir_1P", True)])
def test_sam_couplings(oracle_lib, case, dirichlet):
    g = gold("sam_refs.json")["cases"][case]
    m = sam_model(lambda: oracle_lib.OracleModel(2), dirichlet)
    IA, JA = m.pattern()
    rows = [list(JA[IA[j]:IA[j + 1]] + 1) for j in range(len(IA) - 1)]
    assert rows == g["couplings"]
    madof, meqn = m.sam()
    if "equations" in g:
        for node, eq in g["equations"]["node_eq"]:
            assert max(int(meqn[madof[node - 1] - 1]), 0) == eq
    else:
        assert list(meqn) == list(range(1, len(meqn) + 1))


@pytest.mark.parametrize("case,dirichlet", [("sam_2D_singlebasis_2P", False),
                                            ("sam_2D_singlebasis_dir_2P", True)])
def test_two_patch_sam_couplings(oracle_lib, case, dirichlet):
    g = gold("sam_refs.json")["cases"][case]
    p1 = W.box_patch(2, 1, 1, size=(0.5, 1.0))
    p2 = W.box_patch(2, 1, 1, origin=(0.5, 0.0, 0.0), size=(0.5, 1.0))
    for p in (p1, p2):
        p.kind = 1
    if dirichlet:
        p2.dirichlet = [(2, 1, 1.0)]
    m = oracle_lib.OracleModel(2)
    W.load_into(m, [p1, p2], [tuple(g["connection"])])
    m.preprocess()
    IA, JA = m.pattern()
    assert [list(JA[IA[j]:IA[j + 1]] + 1) for j in range(len(IA) - 1)] == g["couplings"]
    madof, meqn = m.sam()
    eqs = g.get("equations", {}).get("node_eq", [[n, n] for n in range(1, 7)])
    for node, eq in eqs:
        assert max(int(meqn[madof[node - 1] - 1]), 0) == eq


def test_oracle_poisson_converges_to_manufactured_solution(oracle_lib):
    """Global sanity of the restated assembly: -lap u = 2 pi^2 sin sin on the
    unit square; the spline solution converges at O(h^3) in the L2 sense."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    errs = []
    for nel in (8, 16):
        pts, ng = W.config1(nel=nel)
        pts[0].noise = None
        pts[0].source = 2 * np.pi ** 2
        m = oracle_lib.OracleModel(ng)
        W.load_into(m, pts)
        s = m.preprocess()
        m.assemble(1)
        A, b = m.system()
        IA, JA = m.pattern()
        K = sp.csc_matrix((A, JA, IA), shape=(s["neq"],) * 2)
        x = sla.spsolve(K, b)
        madof, meqn = m.sam()
        u = np.zeros(s["ndof"])
        u[meqn > 0] = x[meqn[meqn > 0] - 1]
        X = pts[0].coefs
        errs.append(np.abs(u - np.sin(np.pi * X[:, 0]) * np.sin(np.pi * X[:, 1])).max())
    assert errs[1] < errs[0] / 3.5
