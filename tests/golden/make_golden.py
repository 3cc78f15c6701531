"""Extract golden vectors from IFEM's own unit tests into small JSON fixtures.

Run in a checkout that has the IFEM sources (default /root/reference, or the
path given as the first argument).  The fixtures are committed, so the test
suite never needs the IFEM sources.  Every value is copied from an IFEM test
file or test data file named in the fixture's "source" field.
"""
from __future__ import annotations

import json
import os
import re
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
OUT = os.path.dirname(os.path.abspath(__file__))


def read(rel: str) -> str:
    with open(os.path.join(REF, rel)) as f:
        return f.read()


def numbers(text: str) -> list[float]:
    return [float(x) for x in re.findall(r"-?\d+\.\d*(?:[eE][-+]?\d+)?|-?\d+(?:[eE][-+]?\d+)?", text)]


def block(text: str, start: str, open_ch="{", close_ch="}") -> str:
    """Balanced-brace block that follows the first occurrence of `start`."""
    i = text.index(start)
    j = text.index(open_ch, i)
    depth = 0
    for k in range(j, len(text)):
        if text[k] == open_ch:
            depth += 1
        elif text[k] == close_ch:
            depth -= 1
            if depth == 0:
                return text[j:k + 1]
    raise ValueError(start)


def gauss_tables():
    src = "src/Utility/GaussQuadrature.C"
    t = read(src)
    out = {"source": src, "rules": {}}
    for n in range(1, 11):
        b = block(t, f"static double G{n}[2][{n}]")
        vals = numbers(b)
        assert len(vals) == 2 * n, (n, len(vals))
        out["rules"][str(n)] = {"xi": vals[:n], "w": vals[n:]}
    return out


def sam_refs():
    out = {"source": "src/LinAlg/Test/TestSAM.C:62-96, :133-176 + refdata", "cases": {}}
    for name, xinp in [("sam_2D_singlebasis_1P", "sam_2D_1P.xinp"),
                       ("sam_2D_singlebasis_dir_1P", "sam_2D_dir_1P.xinp"),
                       ("sam_2D_singlebasis_2P", "sam_2D_2P.xinp"),
                       ("sam_2D_singlebasis_dir_2P", "sam_2D_dir_2P.xinp")]:
        rel = f"src/LinAlg/Test/refdata/{name}.ref"
        vals = [int(x) for x in read(rel).split()]
        rows, k = [], 0
        while k < len(vals):
            n = vals[k]
            rows.append(vals[k + 1:k + 1 + n])
            k += 1 + n
        out["cases"][name] = {"ref": rel, "xinp": f"src/LinAlg/Test/refdata/{xinp}",
                              "couplings": rows}
    # equation checks of TestSAM.SingleBasisDirichlet1P: nodes 3,6,9 prescribed
    out["cases"]["sam_2D_singlebasis_dir_1P"]["equations"] = {
        "node_eq": [[1, 1], [2, 2], [3, 0], [4, 3], [5, 4], [6, 0], [7, 5], [8, 6], [9, 0]]}
    # two bilinear patches of square2.g2 ([0,0.5]x[0,1] and [0.5,1]x[0,1]),
    # <connection master="1" medge="2" slave="2" sedge="1"/>; the Dirichlet
    # variant prescribes edge 2 of patch 2 (TestSAM.SingleBasisDirichlet2P:
    # equations 1..4 for nodes 1..4, none for nodes 5, 6)
    for name in ("sam_2D_singlebasis_2P", "sam_2D_singlebasis_dir_2P"):
        out["cases"][name]["geometry"] = "src/LinAlg/Test/refdata/square2.g2"
        out["cases"][name]["connection"] = [1, 2, 2, 1, 0]
    out["cases"]["sam_2D_singlebasis_dir_2P"]["equations"] = {
        "node_eq": [[1, 1], [2, 2], [3, 3], [4, 4], [5, 0], [6, 0]]}
    return out


def equal_order_operators():
    src = "Apps/Utils/Test/TestEqualOrderOperators.C"
    t = read(src)
    lap = t[t.index('TEST_CASE("TestEqualOrderOperators.Laplacian")'):]
    def mat(name, text):
        return numbers(block(text, f"const Real2DMat {name}"))
    # MyElement's constructor sets dNdX(i,j) = v and N(i) = v
    ctor = block(t, "MyElement() : FiniteElement(2)")
    dNdX = [[0.0, 0.0], [0.0, 0.0]]
    for i, j, v in re.findall(r"dNdX\((\d),(\d)\)\s*=\s*([-\d.]+)", ctor):
        dNdX[int(i) - 1][int(j) - 1] = float(v)
    N = [0.0, 0.0]
    for i, v in re.findall(r"\bN\((\d)\)\s*=\s*([-\d.]+)", ctor):
        N[int(i) - 1] = float(v)
    return {"source": src, "dNdX": dNdX, "N": N,
            "laplacian_scalar": mat("EM_scalar_ref", lap),
            "laplacian_multi": mat("EM_multi_ref", lap),
            "laplacian_stress": mat("EM_stress_ref", lap),
            "laplacian_coeff_vec": mat("EM_coeff_refv", lap)}


def jacobian3d():
    src = "src/Utility/Test/TestCoordinateMapping.C"
    t = read(src)
    sec = t[t.index('TEST_CASE("TestCoordinateMapping.Jacobian3D")'):]
    dndx = numbers(block(sec, "const double dndx[]"))
    # the test iterates dNdX (8 x 3) in storage order, i.e. column by column
    return {"source": src + ":357-392",
            "refine": 3, "param": [0.25, 0.25, 0.25], "element": 2,
            "det": 1.0, "dNdX_column_major": dndx}


def spline_surface():
    src = "src/Utility/Test/TestSplineUtils.C"
    t = read(src)
    sec = t[t.index('TEST_CASE("TestSplineUtils.ExtractBasisSurface")'):]
    N = numbers(block(sec, "const double Nref[]"))
    dN = numbers(block(sec, "const double dNdUref[4][2]"))
    return {"source": src + ":98-162", "param": [0.3, 0.3], "N": N,
            "dNdU": [dN[2 * i:2 * i + 2] for i in range(4)]}


def elm_nodes():
    src = "src/ASM/Test/TestASMs3D.C"
    t = read(src)
    sec = t[t.index('TEST_CASE("TestASMs3D.ElmNodes")'):]
    ref = block(sec, "const auto ref =")
    proj = block(sec, "const auto ref_proj =")
    def rows(b):
        return [[int(x) for x in numbers(r)] for r in re.findall(r"std::array\{([^}]*)\}", b)]
    return {"source": src + ":302-326 (ASM3DTests.h:192-223)", "linear": rows(ref),
            "quadratic": rows(proj)}


def gauss_test():
    src = "src/Utility/Test/TestGaussQuadrature.C"
    t = read(src)
    assert "1e-14" in t and "1e-7" in t
    return {"source": src + ":20-36", "rel_tol": 1e-14, "rel_tol_10": 1e-7}


def main():
    fixtures = {
        "gauss_tables.json": gauss_tables(),
        "gauss_test.json": gauss_test(),
        "sam_refs.json": sam_refs(),
        "equal_order_operators.json": equal_order_operators(),
        "jacobian3d.json": jacobian3d(),
        "spline_surface.json": spline_surface(),
        "elm_nodes.json": elm_nodes(),
    }
    for name, data in fixtures.items():
        with open(os.path.join(OUT, name), "w") as f:
            json.dump(data, f, indent=1)
        print("wrote", name)


if __name__ == "__main__":
    main()
