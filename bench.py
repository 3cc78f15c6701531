#!/usr/bin/env python
"""Benchmark: elements/s assembled for 3D linear elasticity on one NURBS patch,
p=2, 24^3 elements, 3x3x3 Gauss points (E=1, nu=0.3, clamped w=0, unit
traction on w=1) -- the IFEM element-integration + assembly path on one GPU.

One step = one full assembly of that model (basis tables, every element's
stiffness and load, Neumann faces, scatter into the compressed-column
system), inputs resident on the device; `value` is elements/s of those
steps.  `e2e` repeats the step through the C ABI with host buffers: the
control net is uploaded from pinned memory and the assembled matrix values
and right-hand side are copied back to pinned host memory inside the timed
region (each step's copy overlaps the next step's assembly; the clock stops
when the last copy has landed).  The `solve` object holds the second half of the metric: wall time to
the FP64 relative residual 1e-10 on the 64^3 p=3 log-normal Poisson system,
plain Jacobi mixed-precision PCG against flexible CG with the Kronecker
preconditioner and with the learned coarse correction (trained in the run,
evaluated on a held-out field).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]
                  [--precision split|fp64] [--solve-nel 64|0]

--impl reference times the reference algorithm on the host cores: IFEM's
ASMs3D::integrate + SAM/assemSparse scatter restated in C++ (oracle/), with
IFEM's OpenMP stripe colouring over all host threads.  Under torchrun every
rank runs an independent replica (the path has no data exchange; replicas
only) and rank 0 prints the line.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NEL = 24
TC_TRAFFIC_24 = 504.0e6  # bytes per launch of the tensor-core element kernel at 24^3 (ncu)
WORKLOAD = "3D linear elasticity, 1 NURBS patch, p=2, 24^3 elements, 3x3x3 Gauss"
METRIC = "elements/s assembled; time to 1e-10 residual, learned vs plain PCG, 1 GB300"


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = f"/tmp/ifemgpu_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.remove(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)),
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_info():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_baseline(patches, ng, threads, budget_s=20.0):
    """The reference algorithm (oracle/, IFEM's integrate + assemSparse restated)
    on `threads` host threads: full assemblies of the model until ~budget_s."""
    import oracle
    orc = oracle.OracleModel(ng)
    from ifem_gb300 import workloads as W
    W.load_into(orc, patches)
    s = orc.preprocess()
    t0 = time.perf_counter()
    orc.assemble(threads)
    first = time.perf_counter() - t0
    reps = max(1, min(5, int(budget_s / max(first, 1e-3))))
    t0 = time.perf_counter()
    for _ in range(reps):
        orc.assemble(threads)
    dt = (time.perf_counter() - t0) / reps
    return s["nel"] / dt, dt, reps, s


# inner reduction of the FP32 iterations per FP64 refinement step for the
# Poisson solve: 3e-6 needs two refinement steps to 1e-10 (1e-4 needs three
# and restarts the Krylov space once more), the same for every method timed
INNER_RTOL = 3e-6

SOLVE_WORKLOAD = ("3D Poisson, 1 B-spline patch, p=3, 64^3 elements, 4x4x4 Gauss, "
                  "log-normal conductivity (GRF sigma 1, correlation 0.1), u=0 on all faces")


def run_solve(args, G, W):
    """Time to the FP64 relative residual 1e-10 on the p=3 log-normal Poisson
    system: plain Jacobi mixed-precision PCG, flexible CG with the Kronecker
    preconditioner, and with the learned coarse correction on top (trained here
    on pairs from seeded conductivity fields, evaluated on a held-out field).
    Each solve is timed on the wall clock around the C-ABI call (device work,
    the FP64 solution copied to host memory) and on device events."""
    t0 = time.perf_counter()
    patches, ng = W.config4(nel=args.solve_nel)
    sim = G.SIM(n_gauss=ng, ke_precision=G.KE_SPLIT_TF32)
    W.load_into(sim, patches)
    sz = sim.preprocess()
    setup_s = time.perf_counter() - t0
    pts = patches[0].coefs[:, :3]
    # assembly of this system (tensor-core Poisson kernel, p = 3): device time
    asm_ms = []
    for _ in range(4):
        sim.assembleSystem()
        asm_ms.append(sim.assembly_stats()[0])
    asm_launches = sim.kernel_launches
    # training: plain-PCG iterates of seeded fields, up to 20,000 pairs
    sim.learn_setup(coarse_cells=args.coarse_cells, hidden=256, capacity=20000, seed=2,
                    field_inputs=1)
    t0 = time.perf_counter()
    seeds = 0
    for s in range(args.train_seeds):
        sim.update_field(1, G.FIELD_LOG_KAPPA,
                         W.gaussian_field_3d(np.random.default_rng(W.BASE_SEED + 500 + s), pts))
        sim.assembleSystem()
        pairs = sim.learn_collect(stride=1, rtol=1e-6)
        seeds += 1
        if pairs >= 20000:
            break
    collect_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    loss = sim.learn_train(epochs=30, batch=128, lr=1e-3, seed=5)
    train_s = time.perf_counter() - t0
    mse_train = sim.learn_evaluate()
    # held-out field: the configuration's own seed
    sim.update_field(1, G.FIELD_LOG_KAPPA, patches[0].log_kappa)
    sim.assembleSystem()
    sim.learn_clear()
    sim.learn_collect(stride=1, rtol=1e-6)
    mse_held = sim.learn_evaluate()
    out = {"workload": SOLVE_WORKLOAD, "neq": sz.neq, "nnz": sz.nnz, "rtol": 1e-10,
           "inner": f"FP32 with FP64 residual refinement (inner reduction {INNER_RTOL:g})",
           "setup_s": setup_s,
           "assembly_ms": float(np.median(asm_ms[1:])), "assembly_launches": asm_launches,
           "assembly_elements_per_s": sz.nel / (float(np.median(asm_ms[1:])) * 1e-3)}
    xs = {}
    for key, meth, pre in (("plain_pcg", G.PCG_MIXED, G.PRECOND_JACOBI),
                           ("kronecker_fcg", G.PCG_MIXED, G.PRECOND_KRONECKER),
                           ("learned_fcg", G.FCG_LEARNED, G.PRECOND_KRONECKER),
                           ("learned_jacobi_fcg", G.FCG_LEARNED, G.PRECOND_JACOBI)):
        for _ in range(2):                               # capture and warm up
            sim.solveSystem(method=meth, rtol=1e-10, precond=pre, inner_rtol=INNER_RTOL,
                            check=False)
        walls, dev = [], []
        for _ in range(args.solve_reps):
            t0 = time.perf_counter()
            x, info = sim.solveSystem(method=meth, rtol=1e-10, precond=pre,
                                      inner_rtol=INNER_RTOL, check=False)
            walls.append((time.perf_counter() - t0) * 1e3)
            dev.append(info.device_ms)
        xs[key] = x
        out[key] = {"wall_ms": float(np.median(walls)), "device_ms": float(np.median(dev)),
                    "inner_iters": info.inner_iters, "outer_iters": info.outer_iters,
                    "relres": info.relres, "fallbacks": info.fallbacks}
    ref = xs["plain_pcg"]
    for key in xs:
        out[key]["max_rel_diff_vs_plain"] = float(np.abs(xs[key] - ref).max() / np.abs(ref).max())
    out["learned_training"] = {"seeds": seeds, "pairs": pairs,
                               "coarse_unknowns": args.coarse_cells and (args.coarse_cells + 1) ** 3,
                               "hidden": 256, "epochs": 30, "final_batch_loss": loss,
                               "mse_train": mse_train, "mse_held_out": mse_held,
                               "collect_s": collect_s, "train_s": train_s}
    p = out["plain_pcg"]["wall_ms"]
    out["speedup_vs_plain_pcg"] = {k: p / out[k]["wall_ms"] for k in
                                   ("kronecker_fcg", "learned_fcg", "learned_jacobi_fcg")}
    out["learned_gain_over_kronecker"] = (out["kronecker_fcg"]["wall_ms"]
                                          / out["learned_fcg"]["wall_ms"])
    return out


def run_assembly_64(args, G, W):
    """The elasticity model at 64^3 elements (262,144 elements, 849,420
    equations, 301 M matrix entries): preprocessing time of the library (host
    numbering and pattern), elements/s of device-resident assemblies (the
    matrix alone, 2.4 GB, is larger than L2), and the time to the FP64
    relative residual 1e-10 with plain mixed PCG and with Kronecker FCG."""
    t0 = time.perf_counter()
    patches, ng = W.config2(nel=64)
    sim = G.SIM(n_gauss=ng, ke_precision=G.KE_SPLIT_TF32)
    W.load_into(sim, patches)
    sz = sim.preprocess()
    pre_s = time.perf_counter() - t0
    for _ in range(2):
        sim.assembleSystem()
    ts, vs = [], []
    for _ in range(args.steps):
        sim.assembleSystem()
        t, v, _ = sim.assembly_stats()
        ts.append(t)
        vs.append(v)
    ms = float(np.median(ts))
    out = {"workload": "3D linear elasticity, 1 NURBS patch, p=2, 64^3 elements, 3x3x3 Gauss",
           "nel": sz.nel, "neq": sz.neq, "nnz": sz.nnz, "preprocess_s": pre_s,
           "ms_per_assembly": ms, "volume_ms": float(np.median(vs)),
           "elements_per_s": sz.nel / (ms * 1e-3), "steps": args.steps}
    for key, pre in (("solve_plain_pcg", G.PRECOND_JACOBI),
                     ("solve_kronecker_fcg", G.PRECOND_KRONECKER)):
        sim.solveSystem(method=G.PCG_MIXED, rtol=1e-10, precond=pre, check=False)
        t0 = time.perf_counter()
        x, info = sim.solveSystem(method=G.PCG_MIXED, rtol=1e-10, precond=pre, check=False)
        out[key] = {"wall_ms": (time.perf_counter() - t0) * 1e3, "device_ms": info.device_ms,
                    "inner_iters": info.inner_iters, "outer_iters": info.outer_iters,
                    "relres": info.relres}
    del sim
    return out


def run_reference(args):
    world, rank, _ = dist_info()
    if rank != 0:
        return
    from ifem_gb300 import workloads as W
    patches, ng = W.config2(nel=NEL)
    threads = os.cpu_count() or 1
    import oracle
    orc = oracle.OracleModel(ng)
    W.load_into(orc, patches)
    s = orc.preprocess()
    for _ in range(max(1, min(args.warmup, 1))):
        orc.assemble(threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        orc.assemble(threads)
        times.append(time.perf_counter() - t0)
    dt = float(np.mean(times))
    value = s["nel"] / dt
    sample = (f"full assembly of the {s['nel']}-element model per step "
              f"(IFEM integrate + assemSparse restated in C++, OpenMP stripe colouring)")
    line = {"metric": METRIC, "value": value, "unit": "elements/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded NURBS patch)",
            "config": {"workload": WORKLOAD, "nel": s["nel"], "neq": s["neq"], "nnz": s["nnz"],
                       "threads": threads},
            "cpu_baseline": {"value": value, "unit": "elements/s", "cores": threads,
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "elements/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def accuracy_vs_fp64(G, W, sim, patches, ng, device):
    """The split-precision system of the benchmark against the FP64 assembly of
    the same model (IFEMGPU_KE_FP64, equal to the oracle and to IFEM's own
    assembly within 1e-12 in the tests): max-norm error relative to max|K|,
    per-entry relative error of the entries above 1e-3 max|K|, right-hand
    side error relative to max|b|."""
    sim.assembleSystem()
    K, b = sim.matrix_values(), sim.rhs()
    ref = G.SIM(n_gauss=ng, ke_precision=G.KE_FP64, device=device)
    W.load_into(ref, patches)
    ref.preprocess()
    ref.assembleSystem()
    Kr, br = ref.matrix_values(), ref.rhs()
    scale = np.abs(Kr).max()
    big = np.abs(Kr) > 1e-3 * scale
    per = np.abs(K[big] - Kr[big]) / np.abs(Kr[big])
    return {"reference": "FP64 assembly of the same model",
            "max_err_rel_to_max": float(np.abs(K - Kr).max() / scale),
            "per_entry_rel_max": float(per.max()), "per_entry_rel_median": float(np.median(per)),
            "entries_compared": int(big.sum()),
            "rhs_err_rel_to_max": float(np.abs(b - br).max() / np.abs(br).max())}


def run_gpu(args):
    import torch
    world, rank, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from ifem_gb300 import build as gbuild
    from ifem_gb300 import ifemgpu as G
    from ifem_gb300 import workloads as W
    gbuild.ensure_built()
    ke = G.KE_SPLIT_TF32 if args.precision == "split" else G.KE_FP64
    patches, ng = W.config2(nel=NEL)
    sim = G.SIM(n_gauss=ng, ke_precision=ke, device=local)
    W.load_into(sim, patches)
    sz = sim.preprocess()
    stream = torch.cuda.ExternalStream(sim.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")   # 256 MB > 129 MB L2
    for _ in range(args.warmup):
        sim.assembleSystem(sync=False)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- device-resident steps -------------------------------------------
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    vol_ms = []
    barrier()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()                         # evict L2 between steps (untimed)
                starts[i].record(stream)
            sim.assembleSystem(sync=False)
            with torch.cuda.stream(stream):
                ends[i].record(stream)
            _, v, _ = sim.assembly_stats()            # synchronises; volume-pass time
            vol_ms.append(v)
        barrier()
        wall = time.perf_counter() - wall0
    step_ms = float(np.mean([s.elapsed_time(e) for s, e in zip(starts, ends)]))
    launches = sim.kernel_launches * args.steps
    clocks = clk.summary()

    # ---- end-to-end through the C ABI with host buffers -----------------------
    coefs_np = torch.from_numpy(np.ascontiguousarray(patches[0].coefs,
                                                     dtype=np.float64)).pin_memory().numpy()
    # two pinned host buffers per result: step i's copy (device snapshot, then
    # D2H on the copy stream) overlaps step i+1's assembly
    Kh = [torch.empty(sz.nnz, dtype=torch.float64).pin_memory().numpy() for _ in range(2)]
    bh = [torch.empty(sz.neq, dtype=torch.float64).pin_memory().numpy() for _ in range(2)]
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        sim.update_coefs(1, coefs_np)                 # H2D of the step's input
        sim.assembleSystem(sync=False)
        sim.copy_system_async(Kh[i % 2], bh[i % 2])   # D2H of the step's result
    sim.copy_wait()                                   # every step's system is in host memory
    barrier()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    h2d = coefs_np.nbytes
    d2h = 8 * (sz.nnz + sz.neq)

    # ---- max over ranks ----------------------------------------------------
    if world > 1:
        t = torch.tensor([step_ms, e2e_ms, float(np.mean(vol_ms))], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        step_ms, e2e_ms, vmax = t.tolist()
    else:
        vmax = float(np.mean(vol_ms))

    if rank == 0:
        hbm, bf16, src = measured_peaks()
        nnz = sz.nnz
        # compulsory bytes of one assembly: write every matrix value once (FP64)
        # and read its row index once, plus the right-hand side
        traffic_alg = nnz * 12 + 4 * (sz.neq + 1) + 8 * sz.neq
        achieved = traffic_alg / (vmax * 1e-3) / 1e9
        nq, ndof_e, ns = 27, 81, 6     # p=2 elasticity: Gauss points, element DOFs, stresses
        flops_el = 2 * nq * (ns * ndof_e ** 2 + ns ** 2 * ndof_e)
        value = world * sz.nel / (step_ms * 1e-3)
        cpu_v, cpu_dt, reps, _ = cpu_baseline(patches, ng, os.cpu_count() or 1,
                                              budget_s=args.cpu_budget)
        line = {
            "metric": METRIC, "value": value, "unit": "elements/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32-split" if ke == G.KE_SPLIT_TF32 else "f64",
            "data": "synthetic (seeded NURBS patch, BASE_SEED+2)",
            "config": {"workload": WORKLOAD, "nel": sz.nel, "neq": sz.neq, "nnz": nnz,
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "l2": "flushed between steps (256 MB write, untimed)",
                       "ke_precision": args.precision},
            "e2e": {"value": world * sz.nel / (e2e_ms * 1e-3), "unit": "elements/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": e2e_ms},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm,
                         # dram__bytes_read.sum + dram__bytes_write.sum of one
                         # launch (one 24^3 assembly), ncu capture of this kernel
                         # on this workload; None for other sizes
                         "traffic": TC_TRAFFIC_24 if NEL == 24 and ke == G.KE_SPLIT_TF32
                         else None,
                         "kernel": "volume integration + scatter passes",
                         "kernel_ms": vmax, "algorithmic_bytes": traffic_alg,
                         "peak_source": src},
            "roofline_tensor": {
                "bound": "tensor", "achieved": flops_el * sz.nel / (vmax * 1e-3) / 1e12,
                "peak": bf16, "unit": "TFLOP/s",
                "frac": flops_el * sz.nel / (vmax * 1e-3) / 1e12 / bf16,
                "flops_per_element": flops_el,
                "note": "element stiffness contraction 2 nq (ns ndof^2 + ns^2 ndof), ns = 6, "
                        "counted once although 3xTF32 issues three MMAs per product; peak = "
                        "measured dense bf16 rate (TF32 runs at half of it)"},
            "cpu_baseline": {"value": cpu_v, "unit": "elements/s", "cores": os.cpu_count(),
                             "kind": "port",
                             "sample": f"{reps} full assemblies of the same model "
                                       f"({cpu_dt * 1e3:.0f} ms each)"},
            "gpu_launches": launches,
            "clocks": clocks,
            "wall_s_timed_region": wall,
        }
        if ke == G.KE_SPLIT_TF32:
            line["accuracy"] = accuracy_vs_fp64(G, W, sim, patches, ng, local)
        if args.big:
            line["assembly_64"] = run_assembly_64(args, G, W)
            line["assembly_64"]["speedup_vs_cpu_port_at_24"] = \
                line["assembly_64"]["elements_per_s"] / cpu_v
        if args.solve_nel > 0:
            line["solve"] = run_solve(args, G, W)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--precision", default="split", choices=["split", "fp64"])
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--solve-nel", type=int, default=64,
                    help="elements per direction of the solve leg (0: skip it)")
    ap.add_argument("--solve-reps", type=int, default=3)
    ap.add_argument("--big", type=int, default=1,
                    help="1: also assemble and solve the 64^3 elasticity model (assembly_64)")
    ap.add_argument("--train-seeds", type=int, default=200)
    ap.add_argument("--coarse-cells", type=int, default=8)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
