"""Build recipe of libifemgpu.so (CUDA sm_103a) -- plain nvcc, no cmake.

The translation units are compiled in parallel and linked into
``ifem_gb300/libifemgpu.so`` next to this file (in-tree, git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(HERE, "libifemgpu.so")
OBJDIR = os.path.join(HERE, "_build")

SOURCES = ["host.cpp", "assembly.cu", "solver.cu", "tc_volume.cu", "tc_poisson.cu", "tc_elast3.cu",
           "gather.cu", "learned.cu", "fdprec.cu", "norms.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fopenmp", "-I", INCLUDE]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return "nvcc"


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OBJDIR, os.path.splitext(src)[0] + ".o")
    cmd = [_nvcc(), *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cpp"):
        cmd.insert(1, "-x=cu")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile every CUDA translation unit for sm_103a and link the C-ABI library."""
    os.makedirs(OBJDIR, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    cmd = [_nvcc(), *ARCH, "-shared", "-Xcompiler", "-fopenmp", *objs, "-o", LIB]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


def is_stale() -> bool:
    """True when the library is missing or older than any source or header."""
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return any(os.path.getmtime(d) > t for d in deps)


def ensure_built() -> str:
    return build() if is_stale() else LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
