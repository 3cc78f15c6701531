"""Write tests/golden/ref_systems.npz: global systems assembled by IFEM's own
code (oracle/refmodel.py over oracle/_ref/libifem_ref.so, built from the IFEM
sources).  Runs only where the IFEM sources are present:

    python oracle/ref/build_ref.py && python tests/golden/make_ref_systems.py

Cases (the seeded synthetic models of ifem_gb300/workloads.py):
  c1_poisson2d_p2   2D Poisson p=2, 8x8 elements, all edges fixed, 3x3 Gauss
  c4_poisson3d_p3   3D Poisson p=3, 3^3 elements, log-normal kappa, 4^3 Gauss
  c3_poisson3d_nurbs 3D Poisson p=2 on a perturbed rational patch, 4^3 elements
  c2_elast3d_p2     3D NURBS elasticity p=2, 2^3 elements, face 5 clamped
  c6_poisson3d_mass 3D NURBS Poisson p=2, 4^3 elements, K + 25 M, face 5 fixed
  c7_elast3d_mass   c2 with K + 50 M (Newmark-type effective stiffness)
  c8_connected_poisson   three connected p=2 Poisson cubes, 2^3 elements each, aligned faces
  c9_connected_rotated   the same with every second patch re-parameterised (orientations 5, 6)
  c10_connected_elast    three connected p=2 elasticity cubes, rotated, clamped at x=0
Cases are (patches, n_gauss) or (patches, n_gauss, connections).
Stored per case: IA, JA (0-based compressed columns), A, b (Poisson), MADOF, MEQN.
For the single-patch 3D cases in SECONDARY also a seeded DOF vector u
(key "u") and the secondary solution of u at every Gauss point (key "sec":
Poisson flux, elasticity stress) evaluated with IFEM's utl::Jacobian.
For c0_poisson2d_small (2D Poisson p=2, 4x4 elements) also the text dumps
IFEM's SparseMatrix::dump / StdVector::dump write, in ref_dump/ (FLAT,
MATLAB, MATRIX_MARKET; zero print tolerance 1e-12).
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from ifem_gb300 import workloads as W  # noqa: E402


def cases():
    """name -> (patches, n_gauss); shared with the tests."""
    rng = np.random.default_rng(W.BASE_SEED + 30)
    nurbs = W.perturb(W.box_patch(3, 2, 4), rng, 0.1)
    nurbs.kind = 1
    nurbs.source = 1.0
    nurbs.dirichlet = [(f, 1, 0.0) for f in range(1, 7)]
    mass_p = W.perturb(W.box_patch(3, 2, 4), np.random.default_rng(W.BASE_SEED + 31), 0.1)
    mass_p.kind = 1
    mass_p.source = 1.0
    mass_p.mass = 25.0
    mass_p.dirichlet = [(5, 1, 0.0)]
    elast_m, ng_m = W.config2(nel=2)
    elast_m[0].mass = 50.0
    return {
        "c0_poisson2d_small": W.config1(nel=4),
        "c1_poisson2d_p2": W.config1(nel=8),
        "c6_poisson3d_mass": ([mass_p], 3),
        "c7_elast3d_mass": (elast_m, ng_m),
        "c8_connected_poisson": W.connected_boxes(1, 2, 2, 3, rotated=False),
        "c9_connected_rotated": W.connected_boxes(1, 2, 2, 3, rotated=True),
        "c10_connected_elast": W.connected_boxes(2, 2, 2, 3, rotated=True),
        "c4_poisson3d_p3": W.config4(nel=3, grid=16),
        "c3_poisson3d_nurbs": ([nurbs], 3),
        "c2_elast3d_p2": W.config2(nel=2),
    }


# single-patch cases whose Gauss-point secondary solution is stored
SECONDARY = ("c4_poisson3d_p3", "c3_poisson3d_nurbs", "c2_elast3d_p2")


def secondary_input(patch):
    """The seeded DOF vector whose secondary solution is stored."""
    nf = 1 if patch.kind == 1 else patch.dim
    return np.random.default_rng(W.BASE_SEED + 40).standard_normal(patch.nnod * nf)


def main():
    from oracle import refmodel
    from oracle.ref import build_ref
    if build_ref.build() is None:
        sys.exit("IFEM sources not present: cannot build the reference")
    here = os.path.dirname(os.path.abspath(__file__))
    os.makedirs(os.path.join(here, "ref_dump"), exist_ok=True)
    out = {}
    for name, case in cases().items():
        patches, ng = case[0], case[1]
        conns = case[2] if len(case) > 2 else ()
        dumps = None
        if name == "c0_poisson2d_small":
            dumps = [(f, os.path.join(here, "ref_dump", f"A.{ext}"),
                      os.path.join(here, "ref_dump", f"b.{ext}"))
                     for f, ext in ((1, "flat"), (2, "m"), (3, "mtx"))]
        if conns:
            ref = refmodel.reference_system_multi(patches, conns, ng)
        else:
            ref = refmodel.reference_system(patches[0], ng, dumps=dumps, zero_tol=1e-12)
        for k, v in ref.items():
            if v is not None:
                out[f"{name}/{k}"] = v
        if name in SECONDARY:
            u = secondary_input(patches[0])
            out[f"{name}/u"] = u
            out[f"{name}/sec"] = refmodel.reference_secondary(patches[0], ng, u)
        print(f"{name}: neq {len(ref['IA']) - 1}, nnz {len(ref['A'])}")
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                     "ref_systems.npz"), **out)


if __name__ == "__main__":
    main()
