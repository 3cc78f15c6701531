#!/usr/bin/env python
"""Benchmark: elements/s assembled for 3D linear elasticity on one NURBS patch,
p=2, 64^3 elements (262,144 elements, 849,420 equations, 301 M matrix
entries), 3x3x3 Gauss points, E=1, nu=0.3, clamped w=0, unit traction on w=1
-- the IFEM element-integration + assembly path on one GPU.

One step = one full assembly of that model (basis tables, every element's
stiffness and load, Neumann faces, scatter into the compressed-column
system), inputs resident on the device; `value` is elements/s of those
steps.  The matrix (2.4 GB of FP64 values) is larger than the 129 MB L2, so
no flush is needed between steps.  `e2e` repeats the step through the C ABI
with host buffers: the control net is uploaded from pinned memory and the
assembled matrix values and right-hand side are copied back to pinned host
memory inside the timed region (each step's copy overlaps the next step's
assembly; the clock stops when the last copy has landed).

Extra objects of the GPU line:
  accuracy       the split-precision 64^3 system against the FP64 assembly of
                 the oracle (IFEM's integrate + assemSparse restated on the
                 host), per entry and in the max norm;
  assembly_24    the same model at 24^3 (device-resident, L2 flushed);
  batched_64_patches  64 patches of uneven size and degree, one system per
                 integrand: ms per assembly and kernel launches;
  elasticity_64  time to the FP64 relative residual 1e-10 on the 64^3 system
                 (plain mixed PCG, Kronecker FCG, and the learned two-level
                 step trained on seeded loads, the traction load held out),
                 solutions against the oracle's FP64 PCG solution;
  roofline       the dominant kernel (the element kernel) against the tensor
                 peak; roofline_gather and roofline_assembly the gather and the
                 whole assembly against HBM (events between the captured
                 segments time each phase);
  solve          the second half of the metric: wall time to 1e-10 on the
                 64^3 p=3 log-normal Poisson system, plain Jacobi mixed PCG
                 against flexible CG with the Kronecker preconditioner and with
                 the learned coarse correction (trained in the run, evaluated
                 on a held-out field), each solution against the oracle's FP64
                 reference solution.
  cpu_baseline   the oracle's assembly on the host cores (bounded sample of the
                 same workload), and the CPU solve baselines (scipy SuperLU
                 with IFEM's options on the 2D Poisson model, the oracle's FP64
                 PCG on the 64^3 Poisson system).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

--impl reference times the reference algorithm on the host cores: IFEM's
ASMs3D::integrate + SAM/assemSparse scatter restated in C++ (oracle/), with
IFEM's OpenMP stripe colouring over all host threads, each step the elements
of the first SAMPLE_LAYERS element layers of the 64^3 model scattered into its
full-size matrix.  Under torchrun every rank runs an independent replica (the
path has no data exchange; replicas only) and rank 0 prints the line.
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

NEL = 64
# element layers (of 64) in one step of the host baseline: 32,768 elements
SAMPLE_LAYERS = 8
WORKLOAD = "3D linear elasticity, 1 NURBS patch, p=2, 64^3 elements, 3x3x3 Gauss"
METRIC = "elements/s assembled; time to 1e-10 residual, learned vs plain PCG, 1 GB300"
DATA = "synthetic (seeded NURBS patch: Greville points + U(-0.1h, 0.1h), weights U[0.8, 1.2])"
# dram__bytes_read.sum + dram__bytes_write.sum per element of the dominant
# kernel (the p=2 elasticity element kernel): 4.7 MB + 1,641.7 MB for the
# 64,000 elements of the 40^3 model (one ncu capture), scaled by the element
# count; about 97% of its 26,576-byte element blocks (the rest is still in L2
# when the kernel ends)
TRAFFIC_PER_ELEMENT = 25725


def config_of(s):
    """The `config` object of both arms (identical keys and values)."""
    return {"workload": WORKLOAD, "nel": int(s["nel"]), "neq": int(s["neq"]),
            "nnz": int(s["nnz"])}


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
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
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


def max_over_ranks(values, device):
    """Element-wise maximum of per-rank timings (the slowest replica sets the
    whole-job time); the values themselves on a single process."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


# ---------------------------------------------------------------------------
# host baseline (oracle: the reference algorithm restated; CPU legs only)

def oracle_model(patches, ng):
    import oracle
    from ifem_gb300 import workloads as W
    orc = oracle.OracleModel(ng)
    W.load_into(orc, patches)
    s = orc.preprocess()
    return orc, s


def sample_elements(s):
    """Elements of one host sample: the first SAMPLE_LAYERS element layers."""
    return min(s["nel"], NEL * NEL * SAMPLE_LAYERS)


def cpu_sample_rate(orc, s, threads, reps):
    """elements/s of `reps` bounded samples of the assembly on `threads` host
    threads (IFEM's stripe colouring over the whole patch; every element of
    the first element layers scattered into the full-size matrix)."""
    n = sample_elements(s)
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        orc.assemble(threads, n)
        times.append(time.perf_counter() - t0)
    dt = float(np.mean(times))
    return n / dt, dt, n


SAMPLE_TEXT = ("elements of the first {layers} of 64 element layers ({n} elements) per "
               "sample, scattered into the full 64^3 matrix (IFEM integrate + assemSparse "
               "restated in C++, IFEM's OpenMP stripe colouring over the whole patch)")


def run_reference(args):
    world, rank, _ = dist_info()
    if rank != 0:
        return
    from ifem_gb300 import workloads as W
    patches, ng = W.config2(nel=NEL)
    threads = os.cpu_count() or 1
    orc, s = oracle_model(patches, ng)
    n = sample_elements(s)
    for _ in range(args.warmup):
        orc.assemble(threads, n)
    value, dt, n = cpu_sample_rate(orc, s, threads, args.steps)
    sample = SAMPLE_TEXT.format(layers=SAMPLE_LAYERS, n=n)
    line = {"metric": METRIC, "value": value, "unit": "elements/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": DATA,
            "config": config_of(s),
            "threads": threads,
            "cpu_baseline": {"value": value, "unit": "elements/s", "cores": threads,
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "elements/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def system_errors(K, b, Kr, br):
    """Split-precision system against an FP64 reference of the same model."""
    scale = float(np.abs(Kr).max())
    big = np.abs(Kr) > 1e-3 * scale
    per = np.abs(K[big] - Kr[big]) / np.abs(Kr[big])
    return {"max_err_rel_to_max": float(np.abs(K - Kr).max() / scale),
            "per_entry_rel_max": float(per.max()),
            "per_entry_rel_median": float(np.median(per)),
            "entries_compared": int(big.sum()),
            "rhs_err_rel_to_max": float(np.abs(b - br).max() / np.abs(br).max())}


def rel_err(x, xr):
    return float(np.abs(x - xr).max() / np.abs(xr).max())


# ---------------------------------------------------------------------------
# extra legs of the GPU line

INNER_RTOL = 3e-6  # inner FP32 reduction per FP64 refinement step of the solves
SOLVE_WORKLOAD = ("3D Poisson, 1 B-spline patch, p=3, 64^3 elements, 4x4x4 Gauss, "
                  "log-normal conductivity (GRF sigma 1, correlation 0.1), u=0 on all faces")


def timed_solves(sim, G, methods, reps):
    out, xs = {}, {}
    for key, meth, pre in methods:
        for _ in range(2):                               # capture and warm up
            sim.solveSystem(method=meth, rtol=1e-10, precond=pre, inner_rtol=INNER_RTOL,
                            check=False)
        walls, dev = [], []
        for _ in range(reps):
            t0 = time.perf_counter()
            x, info = sim.solveSystem(method=meth, rtol=1e-10, precond=pre,
                                      inner_rtol=INNER_RTOL, check=False)
            walls.append((time.perf_counter() - t0) * 1e3)
            dev.append(info.device_ms)
        xs[key] = x
        out[key] = {"wall_ms": float(np.median(walls)), "device_ms": float(np.median(dev)),
                    "inner_iters": info.inner_iters, "outer_iters": info.outer_iters,
                    "relres": info.relres, "fallbacks": info.fallbacks}
    return out, xs


def run_solve(args, G, W, threads):
    """Time to the FP64 relative residual 1e-10 on the p=3 log-normal Poisson
    system: plain Jacobi mixed-precision PCG, flexible CG with the Kronecker
    preconditioner, and with the learned coarse correction on top (trained here
    on pairs from seeded conductivity fields, evaluated on a held-out field).
    Each solve is timed on the wall clock around the C-ABI call (device work,
    the FP64 solution copied to host memory) and on device events.  The FP64
    reference solution is the oracle's FP64 Jacobi-PCG to 1e-13 on the oracle's
    FP64 assembly of the same model; the oracle's PCG to 1e-10 on the host
    cores is the CPU solve baseline."""
    t0 = time.perf_counter()
    patches, ng = W.config4(nel=args.solve_nel)
    sim = G.SIM(n_gauss=ng, ke_precision=G.KE_SPLIT_TF32)
    W.load_into(sim, patches)
    sz = sim.preprocess()
    setup_s = time.perf_counter() - t0
    pts = patches[0].coefs[:, :3]
    asm_ms = []
    for _ in range(4):
        sim.assembleSystem()
        asm_ms.append(sim.assembly_stats()[0])
    asm_launches = sim.kernel_launches
    out = {"workload": SOLVE_WORKLOAD, "neq": sz.neq, "nnz": sz.nnz, "rtol": 1e-10,
           "inner": f"FP32 with FP64 residual refinement (inner reduction {INNER_RTOL:g})",
           "setup_s": setup_s,
           "assembly_ms": float(np.median(asm_ms[1:])), "assembly_launches": asm_launches,
           "assembly_elements_per_s": sz.nel / (float(np.median(asm_ms[1:])) * 1e-3)}
    K, b = sim.matrix_values(), sim.rhs()
    # FP64 reference: the oracle's assembly of the same model and its PCG
    ref = {}
    if args.ref_solve:
        orc, s = oracle_model(patches, ng)
        t0 = time.perf_counter()
        orc.assemble(threads)
        ref_asm_s = time.perf_counter() - t0
        Ko, bo = orc.system()
        out["accuracy"] = dict(system_errors(K, b, Ko, bo),
                               reference="oracle FP64 assembly of the same model")
        del K
        t0 = time.perf_counter()
        x10, it10, rr10 = orc.pcg(bo, rtol=1e-10, threads=threads)
        pcg_s = time.perf_counter() - t0
        xref, itr, rrr = orc.pcg(bo, rtol=1e-13, threads=threads, x0=x10)
        ref = {"x": xref, "cpu": {"assembly_s": ref_asm_s, "pcg_1e-10_s": pcg_s,
                                   "pcg_iters": it10, "pcg_relres": rr10,
                                   "threads": threads,
                                   "what": "oracle FP64 Jacobi-PCG to 1e-10 on the host cores"},
               "relres": rrr}
        del orc, Ko
    # training: complement pairs along Kronecker-FCG iterates of seeded
    # fields, up to 20,000 pairs
    sim.learn_setup(coarse_cells=args.coarse_cells, hidden=256, capacity=20000, seed=2,
                    field_inputs=1)
    sim.learn_set_target(G.LEARN_TARGET_COMPLEMENT)
    t0 = time.perf_counter()
    seeds, pairs = 0, 0
    for s_ in range(args.train_seeds):
        sim.update_field(1, G.FIELD_LOG_KAPPA,
                         W.gaussian_field_3d(np.random.default_rng(W.BASE_SEED + 500 + s_), pts))
        sim.assembleSystem()
        pairs = sim.learn_collect(stride=1, rtol=1e-8, precond=G.PRECOND_KRONECKER)
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
    sim.learn_collect(stride=1, rtol=1e-8, precond=G.PRECOND_KRONECKER)
    mse_held = sim.learn_evaluate()
    res, xs = timed_solves(sim, G, (("plain_pcg", G.PCG_MIXED, G.PRECOND_JACOBI),
                                    ("kronecker_fcg", G.PCG_MIXED, G.PRECOND_KRONECKER),
                                    ("learned_fcg", G.FCG_LEARNED, G.PRECOND_KRONECKER)),
                           args.solve_reps)
    # the first learned solve after an assembly also forms the Galerkin
    # coarse matrix R A R^T (the repeated solves above reuse it)
    sim.assembleSystem()
    t0 = time.perf_counter()
    _, info = sim.solveSystem(method=G.FCG_LEARNED, rtol=1e-10, precond=G.PRECOND_KRONECKER,
                              inner_rtol=INNER_RTOL, check=False)
    res["learned_fcg"]["first_after_assembly"] = {
        "wall_ms": (time.perf_counter() - t0) * 1e3, "device_ms": info.device_ms,
        "inner_iters": info.inner_iters}
    out.update(res)
    for key in xs:
        if ref:
            out[key]["rel_err_vs_fp64_reference"] = rel_err(xs[key], ref["x"])
    if ref:
        out["fp64_reference"] = {"what": "oracle FP64 Jacobi-PCG on the oracle's FP64 "
                                         "assembly, relative residual 1e-13",
                                 "relres": ref["relres"]}
        out["cpu_solve"] = ref["cpu"]
    out["learned_training"] = {"seeds": seeds, "pairs": pairs,
                               "coarse_unknowns": args.coarse_cells and (args.coarse_cells + 1) ** 3,
                               "hidden": 256, "epochs": 30, "final_batch_loss": loss,
                               "mse_train": mse_train, "mse_held_out": mse_held,
                               "collect_s": collect_s, "train_s": train_s}
    p = out["plain_pcg"]["wall_ms"]
    out["speedup_vs_plain_pcg"] = {k: p / out[k]["wall_ms"] for k in
                                   ("kronecker_fcg", "learned_fcg")}
    out["speedup_vs_plain_pcg"]["learned_fcg_first_after_assembly"] = (
        p / out["learned_fcg"]["first_after_assembly"]["wall_ms"])
    out["learned_gain_over_kronecker"] = (out["kronecker_fcg"]["wall_ms"]
                                          / out["learned_fcg"]["wall_ms"])
    return out


def run_assembly_24(args, G, W):
    """The headline model at 24^3 elements (13,824 elements; matrix 132 MB, about
    the L2 size, so L2 is flushed between steps)."""
    import torch
    patches, ng = W.config2(nel=24)
    sim = G.SIM(n_gauss=ng, ke_precision=G.KE_SPLIT_TF32)
    W.load_into(sim, patches)
    sz = sim.preprocess()
    stream = torch.cuda.ExternalStream(sim.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(3):
        sim.assembleSystem()
    ts = []
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        sim.assembleSystem(sync=False)
        t, v, _ = sim.assembly_stats()
        ts.append(t)
    ms = float(np.median(ts))
    return {"workload": WORKLOAD.replace("64^3", "24^3"), "nel": sz.nel, "neq": sz.neq,
            "nnz": sz.nnz, "ms_per_assembly": ms, "elements_per_s": sz.nel / (ms * 1e-3),
            "l2": "flushed between steps (256 MB write, untimed)"}


def run_batched(args, G, W):
    """The batched configuration: 64 independent patches of 8^3..32^3
    elements, p = 2 and 3, Poisson and elasticity, assembled as two systems
    (one per integrand, as the patch kinds need different DOF counts); each
    assembly is the basis tables, one element-kernel launch per kernel class
    over all its patches and one gather per (degree, field) class."""
    patches, ng = W.config3()
    out = {}
    for kind, name in ((1, "poisson"), (2, "elasticity")):
        sub = [pc for pc in patches if pc.kind == kind]
        sim = G.SIM(n_gauss=ng, ke_precision=G.KE_SPLIT_TF32)
        W.load_into(sim, sub)
        sz = sim.preprocess()
        for _ in range(3):
            sim.assembleSystem()
        ts = []
        for _ in range(max(3, args.steps // 2)):
            sim.assembleSystem()
            ts.append(sim.assembly_stats()[0])
        ms = float(np.median(ts))
        out[name] = {"patches": len(sub), "nel": sz.nel, "neq": sz.neq, "nnz": sz.nnz,
                     "ms_per_assembly": ms, "elements_per_s": sz.nel / (ms * 1e-3),
                     "kernel_launches": sim.kernel_launches,
                     "degrees": sorted({int(pc.degree[0]) for pc in sub})}
        del sim
    return out


def seeded_loads(W, patch, sam, seed):
    """A smooth random load per displacement component: a Gaussian random
    field (sigma 1, correlation 0.1) at the control points, as nodal values
    of the free equations."""
    rng = np.random.default_rng(seed)
    pts = patch.coefs[:, :3]
    rhs = np.zeros(int(sam.meqn.max()))
    for comp in range(3):
        f = W.gaussian_field_3d(rng, pts, grid=16)
        eq = sam.meqn[sam.madof[:-1] - 1 + comp]
        rhs[eq[eq > 0] - 1] = f[eq > 0]
    return rhs


def run_elasticity_solves(args, G, W, sim, patches, xref):
    """The 64^3 elasticity system to 1e-10: plain mixed PCG, Kronecker FCG
    and, when args.elast_seeds > 0, the learned two-level step on top of the
    Kronecker preconditioner, its network trained on complement pairs of
    Kronecker-FCG solves with seeded smooth random loads (the benchmark's
    traction load is the held-out right-hand side)."""
    res, xs = timed_solves(sim, G, (("plain_pcg", G.PCG_MIXED, G.PRECOND_JACOBI),
                                    ("kronecker_fcg", G.PCG_MIXED, G.PRECOND_KRONECKER)), 1)
    if args.elast_seeds > 0:
        sam = sim.getSAM()
        sim.learn_setup(coarse_cells=args.coarse_cells, hidden=256, capacity=20000, seed=2,
                        field_inputs=0)
        sim.learn_set_target(G.LEARN_TARGET_COMPLEMENT)
        t0 = time.perf_counter()
        seeds, pairs = 0, 0
        for s_ in range(args.elast_seeds):
            rhs = seeded_loads(W, patches[0], sam, W.BASE_SEED + 900 + s_)
            pairs = sim.learn_collect(rhs=rhs, stride=1, rtol=1e-8, precond=G.PRECOND_KRONECKER)
            seeds += 1
            if pairs >= 20000:
                break
        collect_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        loss = sim.learn_train(epochs=30, batch=128, lr=1e-3, seed=5)
        train_s = time.perf_counter() - t0
        mse_train = sim.learn_evaluate()
        sim.learn_clear()
        sim.learn_collect(stride=1, rtol=1e-8, precond=G.PRECOND_KRONECKER)
        mse_held = sim.learn_evaluate()
        r2, x2 = timed_solves(sim, G, (("learned_fcg", G.FCG_LEARNED, G.PRECOND_KRONECKER),), 1)
        res.update(r2)
        xs.update(x2)
        res["learned_training"] = {
            "seeds": seeds, "pairs": pairs, "coarse_unknowns": 3 * (args.coarse_cells + 1) ** 3,
            "hidden": 256, "epochs": 30, "final_batch_loss": loss, "mse_train": mse_train,
            "mse_held_out": mse_held, "collect_s": collect_s, "train_s": train_s,
            "loads": "seeded smooth random nodal loads (Gaussian random field per component); "
                     "held out: the traction load of the benchmark model"}
        res["learned_gain_over_kronecker"] = (res["kronecker_fcg"]["wall_ms"]
                                              / res["learned_fcg"]["wall_ms"])
    if xref is not None:
        for key in xs:
            res[key]["rel_err_vs_fp64_reference"] = rel_err(xs[key], xref)
    return res


# ---------------------------------------------------------------------------

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
    threads = os.cpu_count() or 1
    patches, ng = W.config2(nel=NEL)
    sim = G.SIM(n_gauss=ng, ke_precision=G.KE_SPLIT_TF32, device=local)
    W.load_into(sim, patches)
    t0 = time.perf_counter()
    sz = sim.preprocess()
    preprocess_s = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(sim.stream())
    for _ in range(args.warmup):
        sim.assembleSystem(sync=False)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- device-resident steps (inputs larger than L2) ----------------------
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    vol_ms, elem_ms, gath_ms = [], [], []
    barrier()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                starts[i].record(stream)
            sim.assembleSystem(sync=False)
            with torch.cuda.stream(stream):
                ends[i].record(stream)
            _, v, _ = sim.assembly_stats()            # synchronises; volume-pass time
            e_ms, g_ms = sim.assembly_phases()         # element kernel, gather
            vol_ms.append(v)
            elem_ms.append(e_ms)
            gath_ms.append(g_ms)
        barrier()
        wall = time.perf_counter() - wall0
    step_ms = float(np.mean([s.elapsed_time(e) for s, e in zip(starts, ends)]))
    launches = sim.kernel_launches * args.steps
    clocks = clk.summary()

    # ---- end-to-end through the C ABI with host buffers -----------------------
    coefs_np = torch.from_numpy(np.ascontiguousarray(patches[0].coefs,
                                                     dtype=np.float64)).pin_memory().numpy()
    Kh = [torch.empty(sz.nnz, dtype=torch.float64).pin_memory().numpy() for _ in range(2)]
    bh = [torch.empty(sz.neq, dtype=torch.float64).pin_memory().numpy() for _ in range(2)]
    for i in range(2):                                # touch the pinned pages once
        sim.assembleSystem(sync=False)
        sim.copy_system_async(Kh[i], bh[i])
    sim.copy_wait()
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
    Ksplit, bsplit = Kh[(args.steps - 1) % 2].copy(), bh[(args.steps - 1) % 2].copy()
    del Kh, bh

    # ---- max over ranks ----------------------------------------------------
    step_ms, e2e_ms, vmax, emax, gmax = max_over_ranks(
        [step_ms, e2e_ms, float(np.mean(vol_ms)), float(np.mean(elem_ms)),
         float(np.mean(gath_ms))], "cuda")

    if rank == 0:
        hbm, bf16, src = measured_peaks()
        nnz = sz.nnz
        # compulsory bytes of one assembly: write every matrix value once (FP64)
        # and read its row index once, plus the right-hand side
        traffic_alg = nnz * 12 + 4 * (sz.neq + 1) + 8 * sz.neq
        achieved = traffic_alg / (vmax * 1e-3) / 1e9
        nq, ndof_e, ns = 27, 81, 6     # p=2 elasticity: Gauss points, element DOFs, stresses
        flops_el = 2 * nq * (ns * ndof_e ** 2 + ns ** 2 * ndof_e)
        tflops_el = flops_el * sz.nel / (emax * 1e-3) / 1e12
        gbs_gather = traffic_alg / (gmax * 1e-3) / 1e9
        value = world * sz.nel / (step_ms * 1e-3)
        # host baseline on the same workload (bounded sample), then the oracle's
        # full FP64 assembly as the reference of the accuracy object
        orc, s = oracle_model(patches, ng)
        orc.assemble(threads, sample_elements(s))
        cpu_v, cpu_dt, n_s = cpu_sample_rate(orc, s, threads, args.cpu_reps)
        orc.assemble(threads)
        Ko, bo = orc.system()
        accuracy = dict(system_errors(Ksplit, bsplit, Ko, bo),
                        reference="oracle FP64 assembly of the same model (IFEM's integrate "
                                  "+ assemSparse restated on the host)")
        del Ksplit, Ko
        xref = None
        if args.ref_solve:
            xref, _, _ = orc.pcg(bo, rtol=1e-12, threads=threads)
        del orc
        line = {
            "metric": METRIC, "value": value, "unit": "elements/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32-split", "data": DATA,
            "config": config_of({"nel": sz.nel, "neq": sz.neq, "nnz": nnz}),
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
            "l2": "inputs larger than L2 (2.4 GB matrix), no flush",
            "ke_precision": "3xTF32 tcgen05 element matrices, FP64 assembly sums",
            "e2e": {"value": world * sz.nel / (e2e_ms * 1e-3), "unit": "elements/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": e2e_ms},
            "roofline": {
                "bound": "tensor", "achieved": tflops_el, "peak": bf16, "unit": "TFLOP/s",
                "frac": tflops_el / bf16,
                "traffic": (TRAFFIC_PER_ELEMENT * sz.nel if TRAFFIC_PER_ELEMENT else None),
                "kernel": "k_volume_tc_elast_p2 (element kernel, the dominant kernel)",
                "kernel_ms": emax, "flops_per_element": flops_el,
                "algorithmic": "Ke contraction 2 nq (ns ndof^2 + ns^2 ndof), ns = 6, ndof = 81, "
                               "nq = 27, counted once although 3xTF32 issues three MMAs per "
                               "product",
                "peak_source": src + " (dense bf16 burst; TF32 runs at half of it)"},
            "roofline_gather": {
                "bound": "hbm", "achieved": gbs_gather, "peak": hbm, "unit": "GB/s",
                "frac": gbs_gather / hbm, "kernel": "k_gather<2, 3> (node-wise sums)",
                "kernel_ms": gmax, "algorithmic_bytes": traffic_alg,
                "algorithmic": "compulsory bytes of the scatter: nnz (8 value + 4 row index) "
                               "+ 4 (neq + 1) + 8 neq; the element blocks it reads "
                               "(26,576 B per element) are not counted",
                "peak_source": src},
            "roofline_assembly": {
                "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "kernel": "element kernel + gather (one assembly)",
                "kernel_ms": vmax, "algorithmic_bytes": traffic_alg, "peak_source": src},
            "cpu_baseline": {"value": cpu_v, "unit": "elements/s", "cores": threads,
                             "kind": "port",
                             "sample": f"{args.cpu_reps} samples: " +
                                       SAMPLE_TEXT.format(layers=SAMPLE_LAYERS, n=n_s) +
                                       f", {cpu_dt * 1e3:.0f} ms each"},
            "gpu_launches": launches,
            "clocks": clocks,
            "wall_s_timed_region": wall,
            "preprocess_s": preprocess_s,
            "accuracy": accuracy,
        }
        line["elasticity_64"] = run_elasticity_solves(args, G, W, sim, patches, xref)
        del sim
        line["assembly_24"] = run_assembly_24(args, G, W)
        line["batched_64_patches"] = run_batched(args, G, W)
        if args.solve_nel > 0:
            line["solve"] = run_solve(args, G, W, threads)
            if "cpu_solve" in line["solve"]:
                line["cpu_baseline"]["solve"] = line["solve"]["cpu_solve"]
        line["cpu_baseline"].setdefault("solve", {})
        line["cpu_baseline"]["solve"]["superlu_2d_poisson"] = superlu_baseline(W)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def superlu_baseline(W):
    """scipy's SuperLU with IFEM's options (MMD on A^T + A, diagonal pivot
    threshold 0.001, symmetric mode; SparseMatrix.C:101-104) on the oracle's
    FP64 system of the 2D Poisson model (p=2, 32^2 elements), one host thread."""
    import scipy.sparse as sp
    from scipy.sparse.linalg import splu
    patches, ng = W.config1()
    orc, s = oracle_model(patches, ng)
    orc.assemble(1)
    A, b = orc.system()
    IA, JA = orc.pattern()
    M = sp.csc_matrix((A, JA, IA), shape=(s["neq"], s["neq"]))
    t0 = time.perf_counter()
    lu = splu(M, permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.001,
              options={"SymmetricMode": True})
    x = lu.solve(b)
    dt = time.perf_counter() - t0
    return {"seconds": dt, "neq": s["neq"], "nnz": s["nnz"], "threads": 1,
            "relres": float(np.linalg.norm(b - M @ x) / np.linalg.norm(b))}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--cpu-reps", type=int, default=3)
    ap.add_argument("--solve-nel", type=int, default=64,
                    help="elements per direction of the Poisson solve leg (0: skip it)")
    ap.add_argument("--solve-reps", type=int, default=3)
    ap.add_argument("--ref-solve", type=int, default=1,
                    help="1: FP64 reference solutions and CPU solve baselines by the oracle")
    ap.add_argument("--train-seeds", type=int, default=200)
    ap.add_argument("--coarse-cells", type=int, default=8)
    ap.add_argument("--elast-seeds", type=int, default=60,
                    help="seeded loads for the learned elasticity leg (0: skip it)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
