"""TEST INFRASTRUCTURE ONLY: build recipe of oracle/_ref/libifem_ref.so.

Compiles, with g++ and no build system, the IFEM sources on the assembly
path that do not need GoTools, SuperLU, CBLAS or tinyxml2, straight from the
read-only IFEM tree, together with the harness and stubs in this folder.
Everything written goes under oracle/_ref/ (git-ignored).  The only
configure-time input, src/IFEM.h, is produced from src/IFEM.h.in by
substituting its version string.

The reference objects are compiled with hidden visibility and per-function
sections, so that linking with --gc-sections keeps only what the harness
reaches (SystemMatrix::create and the other factories that would pull in
excluded libraries fall away).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
LIB = os.path.join(OUT, "libifem_ref.so")
IFEM_ROOT = "/root/reference"

# IFEM sources compiled unmodified (paths relative to the IFEM root)
REF_SOURCES = [
    "src/LinAlg/SAM.C",
    "src/ASM/SAMpatch.C",
    "src/LinAlg/SparseMatrix.C",
    "src/LinAlg/SystemMatrix.C",
    "src/LinAlg/MatVec.C",
    "src/LinAlg/DiagMatrix.C",
    "src/ASM/ASMbase.C",
    "src/ASM/ElmMats.C",
    "src/ASM/FiniteElement.C",
    "src/ASM/IntegrandBase.C",
    "src/Utility/CoordinateMapping.C",
    "src/Utility/GaussQuadrature.C",
    "src/Utility/MPC.C",
    "src/Utility/LogStream.C",
    "src/Utility/Tensor.C",
    "src/Utility/Vec3Oper.C",
    "src/Utility/Profiler.C",
    "Apps/Utils/EqualOrderOperators.C",
]
OWN_SOURCES = ["ref_harness.cpp", "ref_stubs.cpp"]


def _includes(gen: str) -> list[str]:
    dirs = [gen] + [os.path.join(IFEM_ROOT, d) for d in
                    ("src", "src/ASM", "src/LinAlg", "src/SIM", "src/Utility", "Apps/Utils")]
    return [f"-I{d}" for d in dirs]


def available() -> bool:
    return os.path.isdir(os.path.join(IFEM_ROOT, "src", "LinAlg"))


def build(force: bool = False) -> str | None:
    """Compile the reference objects and link libifem_ref.so; None without IFEM."""
    if not available():
        return None
    if not force and os.path.exists(LIB):
        return LIB
    gen = os.path.join(OUT, "gen")
    obj = os.path.join(OUT, "obj")
    os.makedirs(gen, exist_ok=True)
    os.makedirs(obj, exist_ok=True)
    with open(os.path.join(IFEM_ROOT, "src", "IFEM.h.in")) as f:
        text = f.read().replace("@IFEM_VERSION_STRING@", "reference")
    with open(os.path.join(gen, "IFEM.h"), "w") as f:
        f.write(text)
    # the public compile definitions of IFEM's library target (CMakeLists.txt:536-540)
    flags = ["-std=c++17", "-O2", "-fPIC", "-ffunction-sections", "-fdata-sections",
             "-DReal=double", "-DepsZ=1.0e-12", "-DPROFILE_LEVEL=3", *_includes(gen)]

    def compile_one(src: str) -> str:
        own = src in OWN_SOURCES
        path = os.path.join(HERE, src) if own else os.path.join(IFEM_ROOT, src)
        out = os.path.join(obj, ("own_" if own else "ref_") +
                           os.path.splitext(os.path.basename(src))[0] + ".o")
        vis = [] if own else ["-fvisibility=hidden"]
        cmd = ["g++", *flags, *vis, "-c", path, "-o", out]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"reference build failed for {src}:\n{' '.join(cmd)}\n{res.stderr}")
        return out

    srcs = REF_SOURCES + OWN_SOURCES
    with cf.ThreadPoolExecutor(max_workers=min(16, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    cmd = ["g++", "-shared", "-Wl,--gc-sections", "-Wl,--no-undefined", *objs, "-o", LIB]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"reference link failed:\n{res.stderr[-4000:]}")
    return LIB


if __name__ == "__main__":
    print(build(force=True))


def check_adapter(header: str) -> tuple[bool, str]:
    """g++ -fsyntax-only of the IFEM-side adapter header against IFEM's own
    headers (src/{ASM,LinAlg,SIM,Utility}) and include/ifemgpu.h: every
    function marked override must override a virtual that IFEM declares with
    the same signature.  (ok, compiler output)."""
    repo = os.path.dirname(os.path.dirname(HERE))
    inc = [f"-I{os.path.join(IFEM_ROOT, d)}" for d in
           ("src", "src/ASM", "src/LinAlg", "src/SIM", "src/Utility")]
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-x", "c++", "-DReal=double", "-DepsZ=1e-12",
           f"-I{os.path.join(repo, 'include')}", *inc, header]
    res = subprocess.run(cmd, capture_output=True, text=True)
    return res.returncode == 0, res.stdout + res.stderr
