"""Assemble (and solve) one of the synthetic spline workloads and print the
timings as one JSON line.

  python -m ifem_gb300.run --config 4 --nel 64 --solve both
  python -m ifem_gb300.run --config 3 --kind 2 --colour-passes 1

--config 1  2D Poisson p=2 (sine source with control-point noise)
--config 2  3D NURBS elasticity, p=2 or --degree 3 (clamped w=0, traction on
            w=1; Gauss rule p+1)
--config 3  64 independent patches of uneven size and degree; --kind picks the
            Poisson (1) or the elasticity (2) system
--config 4  3D Poisson p=3 with a log-normal conductivity field
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import ifemgpu as G
from . import workloads as W


def build_model(args):
    if args.config == 1:
        return W.config1(nel=args.nel or 32)
    if args.config == 2:
        patches, ng = W.config2(nel=args.nel or 24, p=args.degree)
        return patches, (ng if args.degree == 2 else 0)
    if args.config == 3:
        patches, ng = W.config3()
        return [p for p in patches if p.kind == args.kind], ng
    return W.config4(nel=args.nel or 64)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--config", type=int, choices=[1, 2, 3, 4], default=4)
    ap.add_argument("--nel", type=int, default=0, help="elements per direction (0: default)")
    ap.add_argument("--kind", type=int, choices=[1, 2], default=1)
    ap.add_argument("--degree", type=int, choices=[2, 3], default=2,
                    help="spline degree of --config 2")
    ap.add_argument("--precision", choices=["split", "fp64"], default="split")
    ap.add_argument("--colour-passes", type=int, choices=[0, 1, 2], default=0)
    ap.add_argument("--assemblies", type=int, default=3)
    ap.add_argument("--solve", choices=["none", "jacobi", "kronecker", "both"], default="none")
    ap.add_argument("--rtol", type=float, default=1e-10)
    args = ap.parse_args(argv)
    patches, ng = build_model(args)
    t0 = time.perf_counter()
    ke = G.KE_SPLIT_TF32 if args.precision == "split" else G.KE_FP64
    sim = G.SIM(n_gauss=ng, ke_precision=ke, colour_passes=args.colour_passes)
    W.load_into(sim, patches)
    sz = sim.preprocess()
    out = {"config": args.config, "nel": sz.nel, "neq": sz.neq, "nnz": sz.nnz,
           "preprocess_s": time.perf_counter() - t0}
    times = []
    for _ in range(max(1, args.assemblies)):
        sim.assembleSystem()
        times.append(sim.assembly_stats()[0])
    out.update(assembly_ms=float(np.median(times)), kernel_launches=sim.kernel_launches)
    methods = {"jacobi": [G.PRECOND_JACOBI], "kronecker": [G.PRECOND_KRONECKER],
               "both": [G.PRECOND_JACOBI, G.PRECOND_KRONECKER], "none": []}[args.solve]
    for pre in methods:
        x, info = sim.solveSystem(method=G.PCG_MIXED, rtol=args.rtol, precond=pre)
        key = "jacobi" if pre == G.PRECOND_JACOBI else "kronecker"
        out[key] = {"inner_iters": info.inner_iters, "outer_iters": info.outer_iters,
                    "device_ms": info.device_ms, "relres": info.relres}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
