"""ctypes binding of the C ABI in include/ifemgpu.h, with a host-side mirror of
IFEM's simulator vocabulary (``SIM.preprocess``, ``SIM.getSAM``,
``SAM.getEquation``, ``SIM.assembleSystem``, ``SIM.solveSystem``) so that
tests read like IFEM's own unit tests.

The library must be built (``ifem_gb300.build.build()``); loading fails loudly
otherwise -- there is no CPU fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import LIB

# ---- C structures ---------------------------------------------------------


class Options(C.Structure):
    _fields_ = [("device", C.c_int), ("ke_precision", C.c_int), ("n_gauss", C.c_int),
                ("verbose", C.c_int), ("colour_passes", C.c_int)]


class Sizes(C.Structure):
    _fields_ = [("npatch", C.c_int), ("nnod", C.c_int), ("nel", C.c_int), ("ndof", C.c_int),
                ("neq", C.c_int), ("nceq", C.c_int), ("nnz", C.c_int64)]


class Material(C.Structure):
    _fields_ = [("kind", C.c_int), ("kappa", C.c_double), ("source", C.c_double),
                ("source_shape", C.c_int), ("E", C.c_double), ("nu", C.c_double),
                ("body", C.c_double * 3)]


class SolverOptions(C.Structure):
    _fields_ = [("method", C.c_int), ("rtol", C.c_double), ("max_outer", C.c_int),
                ("max_inner", C.c_int), ("inner_rtol", C.c_double), ("precond", C.c_int)]


class SolveInfo(C.Structure):
    _fields_ = [("outer_iters", C.c_int), ("inner_iters", C.c_int), ("relres", C.c_double),
                ("device_ms", C.c_double), ("fallbacks", C.c_int)]


class LearnOptions(C.Structure):
    _fields_ = [("coarse_cells", C.c_int), ("hidden", C.c_int), ("capacity", C.c_int),
                ("seed", C.c_uint), ("field_inputs", C.c_int)]


OK, INVALID_ARG, OUT_OF_MEMORY, SINGULAR_JACOBIAN, NOT_CONVERGED, DEVICE_TIMEOUT, \
    CUDA_ERROR, NOT_READY, UNSUPPORTED = range(9)
STATUS_NAMES = ["OK", "INVALID_ARG", "OUT_OF_MEMORY", "SINGULAR_JACOBIAN", "NOT_CONVERGED",
                "DEVICE_TIMEOUT", "CUDA_ERROR", "NOT_READY", "UNSUPPORTED"]
KE_FP64, KE_SPLIT_TF32 = 0, 1
POISSON, ELASTICITY = 1, 2
SOURCE_CONSTANT, SOURCE_SINE = 0, 1
FIELD_LOG_KAPPA, FIELD_SOURCE_NOISE = 1, 2
PCG_MIXED, PCG_FP64, FCG_LEARNED = 1, 2, 3
PRECOND_JACOBI, PRECOND_KRONECKER = 0, 1
LEARN_TARGET_ERROR, LEARN_TARGET_COMPLEMENT = 0, 1
DUMP_FLAT, DUMP_MATLAB, DUMP_MATRIX_MARKET = 1, 2, 3

# Every symbol include/ifemgpu.h declares (checked by the CPU test suite).
EXPORTS = [
    "ifemgpu_ctx_create", "ifemgpu_ctx_destroy", "ifemgpu_last_error", "ifemgpu_abi_version",
    "ifemgpu_patch_add", "ifemgpu_patch_set_material", "ifemgpu_patch_set_field",
    "ifemgpu_patch_set_mass", "ifemgpu_dump_system", "ifemgpu_write_system", "ifemgpu_patch_connect",
    "ifemgpu_solution_norms", "ifemgpu_secondary_solution",
    "ifemgpu_patch_constrain_face", "ifemgpu_patch_add_neumann", "ifemgpu_preprocess",
    "ifemgpu_get_sizes", "ifemgpu_get_madof", "ifemgpu_get_meqn", "ifemgpu_get_mnpc",
    "ifemgpu_get_pattern", "ifemgpu_assemble", "ifemgpu_copy_matrix", "ifemgpu_copy_rhs",
    "ifemgpu_device_system", "ifemgpu_last_assembly_stats", "ifemgpu_last_assembly_phases",
    "ifemgpu_solve",
    "ifemgpu_copy_system_async", "ifemgpu_copy_wait",
    "ifemgpu_expand_solution", "ifemgpu_patch_update_coefs", "ifemgpu_get_stream",
    "ifemgpu_selftest_tc_gemm", "ifemgpu_solve_noalloc", "ifemgpu_learn_setup",
    "ifemgpu_learn_collect", "ifemgpu_learn_clear", "ifemgpu_learn_set_target", "ifemgpu_learn_train",
    "ifemgpu_learn_evaluate", "ifemgpu_learn_gradients", "ifemgpu_learn_info",
    "ifemgpu_learn_coarse_matrix", "ifemgpu_learn_forward",
    "ifemgpu_learn_get_weights", "ifemgpu_learn_set_weights", "ifemgpu_patch_update_field",
    "ifemgpu_learn_get_pairs", "ifemgpu_apply_preconditioner", "ifemgpu_copy_matrix_bsr",
    "ifemgpu_graph_capture", "ifemgpu_graph_launch", "ifemgpu_debug_waits",
]


class IfemGpuError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES[status] if 0 <= status < 9 else status}: {msg}")
        self.status = status


_lib = None


def load_library(path: str | None = None):
    """Load libifemgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB
    if not os.path.exists(path):
        raise OSError(f"{path} not built: run ifem_gb300.build.build()")
    lib = C.CDLL(path)
    P, I, D, V = C.c_void_p, C.c_int, C.c_double, C.c_void_p
    sig = {
        "ifemgpu_ctx_create": (I, [C.POINTER(P), C.POINTER(Options)]),
        "ifemgpu_ctx_destroy": (None, [P]),
        "ifemgpu_last_error": (C.c_char_p, [P]),
        "ifemgpu_abi_version": (I, []),
        "ifemgpu_patch_add": (I, [P, I, V, V, V, V, I, C.POINTER(I)]),
        "ifemgpu_patch_set_material": (I, [P, I, C.POINTER(Material)]),
        "ifemgpu_patch_set_field": (I, [P, I, I, V]),
        "ifemgpu_patch_set_mass": (I, [P, I, D]),
        "ifemgpu_patch_connect": (I, [P, I, I, I, I, I]),
        "ifemgpu_dump_system": (I, [P, C.c_char_p, C.c_char_p, I, D]),
        "ifemgpu_write_system": (I, [I, V, V, V, V, C.c_char_p, C.c_char_p, I, D]),
        "ifemgpu_solution_norms": (I, [P, V, V, V]),
        "ifemgpu_secondary_solution": (I, [P, I, V, V]),
        "ifemgpu_patch_constrain_face": (I, [P, I, I, I, D]),
        "ifemgpu_patch_add_neumann": (I, [P, I, I, V]),
        "ifemgpu_preprocess": (I, [P]),
        "ifemgpu_get_sizes": (I, [P, C.POINTER(Sizes)]),
        "ifemgpu_get_madof": (I, [P, V]),
        "ifemgpu_get_meqn": (I, [P, V]),
        "ifemgpu_get_mnpc": (I, [P, I, V]),
        "ifemgpu_get_pattern": (I, [P, V, V]),
        "ifemgpu_assemble": (I, [P, I]),
        "ifemgpu_copy_matrix": (I, [P, V]),
        "ifemgpu_copy_rhs": (I, [P, V]),
        "ifemgpu_device_system": (I, [P, V, V, V, V]),
        "ifemgpu_last_assembly_stats": (I, [P, C.POINTER(D), C.POINTER(D),
                                            C.POINTER(C.c_longlong), C.POINTER(I)]),
        "ifemgpu_last_assembly_phases": (I, [P, C.POINTER(D), C.POINTER(D)]),
        "ifemgpu_solve": (I, [P, C.POINTER(SolverOptions), V, C.POINTER(SolveInfo)]),
        "ifemgpu_expand_solution": (I, [P, V, V, D]),
        "ifemgpu_patch_update_coefs": (I, [P, I, V]),
        "ifemgpu_get_stream": (I, [P, C.POINTER(C.c_void_p)]),
        "ifemgpu_selftest_tc_gemm": (I, [V, V, V]),
        "ifemgpu_solve_noalloc": (I, [P, D, I, V, C.POINTER(SolveInfo)]),
        "ifemgpu_graph_capture": (I, [P, C.POINTER(SolverOptions)]),
        "ifemgpu_graph_launch": (I, [P, V, C.POINTER(SolveInfo)]),
        "ifemgpu_debug_waits": (I, [P, C.c_uint, C.c_uint, I, I]),
        "ifemgpu_learn_setup": (I, [P, C.POINTER(LearnOptions)]),
        "ifemgpu_learn_collect": (I, [P, V, V, I, I, D, I, C.POINTER(I)]),
        "ifemgpu_learn_clear": (I, [P]),
        "ifemgpu_learn_set_target": (I, [P, I]),
        "ifemgpu_copy_system_async": (I, [P, V, V]),
        "ifemgpu_copy_wait": (I, [P]),
        "ifemgpu_learn_get_pairs": (I, [P, I, I, V, V]),
        "ifemgpu_apply_preconditioner": (I, [P, I, V, V]),
        "ifemgpu_copy_matrix_bsr": (I, [P, I, C.POINTER(I), C.POINTER(C.c_int64), V, V, V]),
        "ifemgpu_learn_train": (I, [P, I, I, C.c_float, C.c_uint, C.POINTER(C.c_float)]),
        "ifemgpu_learn_evaluate": (I, [P, C.POINTER(C.c_float)]),
        "ifemgpu_learn_gradients": (I, [P, V, V, I, V, C.POINTER(C.c_float)]),
        "ifemgpu_learn_info": (I, [P, C.POINTER(I), C.POINTER(I), C.POINTER(I), C.POINTER(I),
                                   C.POINTER(I)]),
        "ifemgpu_learn_get_weights": (I, [P, V, C.POINTER(I), C.POINTER(C.c_float)]),
        "ifemgpu_learn_set_weights": (I, [P, V, I, C.c_float]),
        "ifemgpu_learn_coarse_matrix": (I, [P, V]),
        "ifemgpu_learn_forward": (I, [P, V, V]),
        "ifemgpu_patch_update_field": (I, [P, I, I, V]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def write_system(colptr, rowidx, values, rhs, matrix_path=None, rhs_path=None,
                 fmt: int = DUMP_MATRIX_MARKET, zero_tol: float = 0.0, lib=None):
    """IFEM's text formats for caller arrays (no context or GPU needed)."""
    L = lib or load_library()
    cp = np.ascontiguousarray(colptr, dtype=np.int32)
    ri = np.ascontiguousarray(rowidx, dtype=np.int32)
    va = np.ascontiguousarray(values, dtype=np.float64)
    b = np.ascontiguousarray(rhs if rhs is not None else np.zeros(len(cp) - 1), dtype=np.float64)
    enc = lambda p: None if p is None else os.fspath(p).encode()
    st = L.ifemgpu_write_system(len(cp) - 1, _ptr(cp), _ptr(ri), _ptr(va), _ptr(b),
                                enc(matrix_path), enc(rhs_path), fmt, float(zero_tol))
    if st != OK:
        raise IfemGpuError(st, "write_system failed")


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def selftest_tc_gemm(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """D = A B^T on the tensor cores (A 128x32, B 96x32 float32)."""
    lib = load_library()
    A = np.ascontiguousarray(A, dtype=np.float32)
    B = np.ascontiguousarray(B, dtype=np.float32)
    assert A.shape == (128, 32) and B.shape == (96, 32)
    D = np.zeros((128, 96), dtype=np.float32)
    st = lib.ifemgpu_selftest_tc_gemm(_ptr(A), _ptr(B), _ptr(D))
    if st != OK:
        raise IfemGpuError(st, "tensor-core self-test failed")
    return D


class SAM:
    """Read-only view of the DOF numbering (IFEM SAM, src/LinAlg/SAM.h)."""

    def __init__(self, madof: np.ndarray, meqn: np.ndarray, colptr: np.ndarray,
                 rowidx: np.ndarray):
        self.madof, self.meqn, self.colptr, self.rowidx = madof, meqn, colptr, rowidx

    def getNoNodes(self) -> int:
        return len(self.madof) - 1

    def getNoEquations(self) -> int:
        return len(self.colptr) - 1

    def getEquation(self, inod: int, ldof: int) -> int:
        """SAM::getEquation (src/LinAlg/SAM.C:746-755): 1-based node and DOF."""
        if inod < 1 or inod > self.getNoNodes() or ldof < 1:
            return -1
        idof = self.madof[inod - 1] + ldof - 1
        if idof >= self.madof[inod]:
            return -2
        ieq = int(self.meqn[idof - 1])
        return ieq if ieq > 0 else 0

    def getDofCouplings(self) -> list[list[int]]:
        """Sorted 1-based coupled equations per equation (SAM::getDofCouplings)."""
        return [list((self.rowidx[self.colptr[j]:self.colptr[j + 1]] + 1).tolist())
                for j in range(self.getNoEquations())]


class SIM:
    """One GPU model: patches, numbering, system (mirrors SIMbase usage)."""

    def __init__(self, n_gauss: int = 4, ke_precision: int = KE_FP64, device: int = 0,
                 verbose: int = 0, colour_passes: int = 0):
        self.lib = load_library()
        self.ctx = C.c_void_p()
        opts = Options(device, ke_precision, n_gauss, verbose, colour_passes)
        st = self.lib.ifemgpu_ctx_create(C.byref(self.ctx), C.byref(opts))
        if st != OK:
            raise IfemGpuError(st, "ifemgpu_ctx_create failed (no CUDA device?)")
        self.sizes = None
        self._patches = []

    def _check(self, st: int):
        if st != OK:
            raise IfemGpuError(st, self.lib.ifemgpu_last_error(self.ctx).decode())

    def close(self):
        if self.ctx:
            self.lib.ifemgpu_ctx_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- model input -------------------------------------------------------
    def add_patch(self, patch) -> int:
        """patch: ifem_gb300.workloads.SplinePatch (degree, ncoef, knots, coefs, rational)."""
        dim = patch.dim
        deg = np.ascontiguousarray(patch.degree, dtype=np.int32)
        nco = np.ascontiguousarray(patch.ncoef, dtype=np.int32)
        kn = [np.ascontiguousarray(k, dtype=np.float64) for k in patch.knots]
        karr = (C.c_void_p * 3)(*[_ptr(k) for k in kn] + [None] * (3 - dim))
        coefs = np.ascontiguousarray(patch.coefs, dtype=np.float64)
        pid = C.c_int()
        self._check(self.lib.ifemgpu_patch_add(self.ctx, dim, _ptr(deg), _ptr(nco),
                                               C.cast(karr, C.c_void_p), _ptr(coefs),
                                               int(patch.rational), C.byref(pid)))
        self._patches.append((patch, kn, coefs))
        return pid.value

    def set_material(self, pid: int, kind: int, kappa=1.0, source=0.0, source_shape=0,
                     E=1.0, nu=0.3, body=(0.0, 0.0, 0.0)):
        m = Material(kind, kappa, source, source_shape, E, nu, (C.c_double * 3)(*body))
        self._check(self.lib.ifemgpu_patch_set_material(self.ctx, pid, C.byref(m)))

    def connect(self, master: int, mface: int, slave: int, sface: int, orient: int = 0):
        """Conforming connection of two patches (SIM3D::connectPatches)."""
        self._check(self.lib.ifemgpu_patch_connect(self.ctx, master, mface, slave, sface, orient))

    def set_mass(self, pid: int, scale: float):
        """K_eff = K + scale * M (consistent mass, EqualOrderOperators::Weak::Mass)."""
        self._check(self.lib.ifemgpu_patch_set_mass(self.ctx, pid, float(scale)))

    def set_field(self, pid: int, which: int, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        self._check(self.lib.ifemgpu_patch_set_field(self.ctx, pid, which, _ptr(v)))

    def constrain_face(self, pid: int, face: int, dofs: int, value: float = 0.0):
        self._check(self.lib.ifemgpu_patch_constrain_face(self.ctx, pid, face, dofs, value))

    def add_neumann(self, pid: int, face: int, values):
        v = np.zeros(3)
        v[:len(values)] = values
        self._check(self.lib.ifemgpu_patch_add_neumann(self.ctx, pid, face, _ptr(v)))

    # ---- preprocessing -------------------------------------------------------
    def preprocess(self):
        self._check(self.lib.ifemgpu_preprocess(self.ctx))
        s = Sizes()
        self._check(self.lib.ifemgpu_get_sizes(self.ctx, C.byref(s)))
        self.sizes = s
        return s

    def getSAM(self) -> SAM:
        s = self.sizes
        madof = np.zeros(s.nnod + 1, dtype=np.int32)
        meqn = np.zeros(s.ndof, dtype=np.int32)
        colptr = np.zeros(s.neq + 1, dtype=np.int32)
        rowidx = np.zeros(max(s.nnz, 1), dtype=np.int32)
        self._check(self.lib.ifemgpu_get_madof(self.ctx, _ptr(madof)))
        self._check(self.lib.ifemgpu_get_meqn(self.ctx, _ptr(meqn)))
        self._check(self.lib.ifemgpu_get_pattern(self.ctx, _ptr(colptr), _ptr(rowidx)))
        return SAM(madof, meqn, colptr, rowidx[:s.nnz])

    def mnpc(self, pid: int) -> np.ndarray:
        patch = self._patches[pid - 1][0]
        nel = int(np.prod([n - p for n, p in zip(patch.ncoef, patch.degree)]))
        nen = int(np.prod([p + 1 for p in patch.degree]))
        out = np.zeros(nel * nen, dtype=np.int32)
        self._check(self.lib.ifemgpu_get_mnpc(self.ctx, pid, _ptr(out)))
        return out.reshape(nel, nen)

    def update_coefs(self, pid: int, coefs: np.ndarray):
        """Asynchronous upload: `coefs` must stay alive until the next sync."""
        assert coefs.flags.c_contiguous and coefs.dtype == np.float64
        self._check(self.lib.ifemgpu_patch_update_coefs(self.ctx, pid, _ptr(coefs)))

    def stream(self) -> int:
        s = C.c_void_p()
        self._check(self.lib.ifemgpu_get_stream(self.ctx, C.byref(s)))
        return s.value or 0

    # ---- assembly / solve ----------------------------------------------------
    def assembleSystem(self, sync: bool = True):
        self._check(self.lib.ifemgpu_assemble(self.ctx, 1 if sync else 0))

    def assembly_stats(self):
        t, v, s, n = C.c_double(), C.c_double(), C.c_longlong(), C.c_int()
        self._check(self.lib.ifemgpu_last_assembly_stats(self.ctx, C.byref(t), C.byref(v),
                                                         C.byref(s), C.byref(n)))
        self.kernel_launches = n.value
        return t.value, v.value, s.value

    def assembly_phases(self):
        """(element-kernel ms, gather ms) of the last assembly."""
        e, g = C.c_double(), C.c_double()
        self._check(self.lib.ifemgpu_last_assembly_phases(self.ctx, C.byref(e), C.byref(g)))
        return e.value, g.value

    def matrix_values(self) -> np.ndarray:
        out = np.zeros(self.sizes.nnz, dtype=np.float64)
        self._check(self.lib.ifemgpu_copy_matrix(self.ctx, _ptr(out)))
        return out

    def rhs(self) -> np.ndarray:
        out = np.zeros(self.sizes.neq, dtype=np.float64)
        self._check(self.lib.ifemgpu_copy_rhs(self.ctx, _ptr(out)))
        return out

    def solution_norms(self, u_dof, per_element: bool = False):
        """(a(u,u), int u.u) and optionally per-element values (nel x 2)."""
        u = np.ascontiguousarray(u_dof, dtype=np.float64)
        tot = np.zeros(2)
        nel = sum(pc.nel for pc, _, _ in self._patches)
        el = np.zeros((nel, 2)) if per_element else None
        self._check(self.lib.ifemgpu_solution_norms(self.ctx, _ptr(u), _ptr(tot),
                                                    _ptr(el) if per_element else None))
        return (tot, el) if per_element else tot

    def secondary_solution(self, pid: int, u_dof, nq: int, ncomp: int):
        """Flux (Poisson) or stress (elasticity) at the Gauss points of patch
        pid: array (nel, nq, ncomp)."""
        u = np.ascontiguousarray(u_dof, dtype=np.float64)
        nel = self._patches[pid - 1][0].nel
        out = np.zeros((nel, nq, ncomp))
        self._check(self.lib.ifemgpu_secondary_solution(self.ctx, pid, _ptr(u), _ptr(out)))
        return out

    def dump_system(self, matrix_path=None, rhs_path=None, fmt: int = DUMP_MATRIX_MARKET,
                    zero_tol: float = 0.0):
        """SIMbase::dumpEqSys: the matrix ("A") and right-hand side ("b") in
        IFEM's text formats (DUMP_FLAT, DUMP_MATLAB, DUMP_MATRIX_MARKET)."""
        enc = lambda p: None if p is None else os.fspath(p).encode()
        self._check(self.lib.ifemgpu_dump_system(self.ctx, enc(matrix_path), enc(rhs_path), fmt,
                                                 float(zero_tol)))

    def matrix_bsr(self, block: int):
        """(browptr, bcolind, blocks[nnzb, block, block]) of the assembled matrix."""
        nb, nnzb = C.c_int(), C.c_int64()
        self._check(self.lib.ifemgpu_copy_matrix_bsr(self.ctx, block, C.byref(nb), C.byref(nnzb),
                                                     None, None, None))
        rp = np.zeros(nb.value + 1, dtype=np.int32)
        ci = np.zeros(nnzb.value, dtype=np.int32)
        vals = np.zeros((nnzb.value, block, block), dtype=np.float64)
        self._check(self.lib.ifemgpu_copy_matrix_bsr(self.ctx, block, C.byref(nb), C.byref(nnzb),
                                                     _ptr(rp), _ptr(ci), _ptr(vals)))
        return rp, ci, vals

    def copy_matrix_into(self, out: np.ndarray):
        assert out.dtype == np.float64 and out.size >= self.sizes.nnz
        self._check(self.lib.ifemgpu_copy_matrix(self.ctx, _ptr(out)))

    def copy_rhs_into(self, out: np.ndarray):
        assert out.dtype == np.float64 and out.size >= self.sizes.neq
        self._check(self.lib.ifemgpu_copy_rhs(self.ctx, _ptr(out)))

    def copy_system_async(self, values: np.ndarray, rhs: np.ndarray | None = None):
        """Snapshot K (and b) and copy them to the host buffers on the copy
        stream; the buffers must stay alive and untouched until copy_wait()."""
        assert values.dtype == np.float64 and values.size >= self.sizes.nnz
        assert rhs is None or (rhs.dtype == np.float64 and rhs.size >= self.sizes.neq)
        self._check(self.lib.ifemgpu_copy_system_async(self.ctx, _ptr(values),
                                                       None if rhs is None else _ptr(rhs)))

    def copy_wait(self):
        self._check(self.lib.ifemgpu_copy_wait(self.ctx))

    def solveSystem(self, method=PCG_MIXED, rtol=1e-10, max_outer=20, max_inner=20000,
                    inner_rtol=1e-4, check=True, precond=PRECOND_JACOBI):
        x = np.zeros(self.sizes.neq, dtype=np.float64)
        o = SolverOptions(method, rtol, max_outer, max_inner, inner_rtol, precond)
        info = SolveInfo()
        st = self.lib.ifemgpu_solve(self.ctx, C.byref(o), _ptr(x), C.byref(info))
        if check:
            self._check(st)
        return x, info

    def graph_capture(self, rtol=1e-10, max_outer=20, max_inner=20000, inner_rtol=1e-4,
                      precond=PRECOND_JACOBI):
        """Captures one assemble -> solve step (mixed-precision PCG / FCG)."""
        o = SolverOptions(PCG_MIXED, rtol, max_outer, max_inner, inner_rtol, precond)
        self._check(self.lib.ifemgpu_graph_capture(self.ctx, C.byref(o)))

    def graph_launch(self, check=True):
        """Replays the captured step: (solution, info)."""
        x = np.zeros(self.sizes.neq, dtype=np.float64)
        info = SolveInfo()
        st = self.lib.ifemgpu_graph_launch(self.ctx, _ptr(x), C.byref(info))
        if check:
            self._check(st)
        return x, info

    def solve_noalloc(self, rtol=1e-10, max_iter=20000, check=True):
        """FP64 Jacobi-PCG through the allocation-free entry point (fixed
        library workspace, at most 65,536 equations)."""
        x = np.zeros(self.sizes.neq, dtype=np.float64)
        info = SolveInfo()
        st = self.lib.ifemgpu_solve_noalloc(self.ctx, rtol, max_iter, _ptr(x), C.byref(info))
        if check:
            self._check(st)
        return x, info, st

    def expand_solution(self, x: np.ndarray, scale: float = 1.0) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        u = np.zeros(self.sizes.ndof, dtype=np.float64)
        self._check(self.lib.ifemgpu_expand_solution(self.ctx, _ptr(x), _ptr(u), scale))
        return u

    def apply_preconditioner(self, r: np.ndarray, precond=PRECOND_KRONECKER) -> np.ndarray:
        r = np.ascontiguousarray(r, dtype=np.float64)
        z = np.zeros(self.sizes.neq, dtype=np.float64)
        self._check(self.lib.ifemgpu_apply_preconditioner(self.ctx, precond, _ptr(r), _ptr(z)))
        return z

    # ---- learned coarse correction -----------------------------------------
    def update_field(self, pid: int, which: int, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        self._check(self.lib.ifemgpu_patch_update_field(self.ctx, pid, which, _ptr(v)))

    def learn_setup(self, coarse_cells=8, hidden=256, capacity=20000, seed=1, field_inputs=0):
        o = LearnOptions(coarse_cells, hidden, capacity, seed, field_inputs)
        self._check(self.lib.ifemgpu_learn_setup(self.ctx, C.byref(o)))
        return self.learn_info()

    def learn_info(self) -> dict:
        nc, nin, nh, npar, pairs = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_int()
        self._check(self.lib.ifemgpu_learn_info(self.ctx, C.byref(nc), C.byref(nin), C.byref(nh),
                                                C.byref(npar), C.byref(pairs)))
        return {"coarse_unknowns": nc.value, "inputs": nin.value, "hidden": nh.value,
                "nparam": npar.value, "pairs": pairs.value}

    def learn_collect(self, rhs=None, xstar=None, stride=1, max_iter=20000, rtol=1e-6,
                      precond=PRECOND_JACOBI) -> int:
        keep = []
        args = []
        for a in (rhs, xstar):
            if a is None:
                args.append(None)
            else:
                v = np.ascontiguousarray(a, dtype=np.float64)
                assert v.size == self.sizes.neq
                keep.append(v)
                args.append(_ptr(v))
        n = C.c_int()
        self._check(self.lib.ifemgpu_learn_collect(self.ctx, args[0], args[1], stride, max_iter,
                                                   rtol, precond, C.byref(n)))
        return n.value

    def learn_coarse_matrix(self) -> np.ndarray:
        """Galerkin coarse matrix R A R^T of the assembled system (dense)."""
        nc = self.learn_info()["coarse_unknowns"]
        Ac = np.zeros((nc, nc), dtype=np.float32)
        self._check(self.lib.ifemgpu_learn_coarse_matrix(self.ctx, _ptr(Ac)))
        return Ac

    def learn_forward(self, rc: np.ndarray) -> np.ndarray:
        """The network's output for a coarse input through the solve's
        tensor-core inference path."""
        rc = np.ascontiguousarray(rc, dtype=np.float32)
        y = np.zeros(self.learn_info()["coarse_unknowns"], dtype=np.float32)
        self._check(self.lib.ifemgpu_learn_forward(self.ctx, _ptr(rc), _ptr(y)))
        return y

    def learn_clear(self):
        self._check(self.lib.ifemgpu_learn_clear(self.ctx))

    def learn_set_target(self, mode):
        """LEARN_TARGET_ERROR (whole coarse error) or LEARN_TARGET_COMPLEMENT
        (the error minus the Kronecker preconditioner's output); forgets the
        stored pairs when the mode changes."""
        self._check(self.lib.ifemgpu_learn_set_target(self.ctx, mode))

    def learn_pairs(self, first=0, count=None):
        info = self.learn_info()
        count = info["pairs"] - first if count is None else count
        X = np.zeros((count, info["inputs"]), dtype=np.float32)
        Y = np.zeros((count, info["coarse_unknowns"]), dtype=np.float32)
        self._check(self.lib.ifemgpu_learn_get_pairs(self.ctx, first, count, _ptr(X), _ptr(Y)))
        return X, Y

    def learn_train(self, epochs=20, batch=256, lr=1e-3, seed=7) -> float:
        loss = C.c_float()
        self._check(self.lib.ifemgpu_learn_train(self.ctx, epochs, batch, lr, seed,
                                                 C.byref(loss)))
        return loss.value

    def learn_evaluate(self) -> float:
        mse = C.c_float()
        self._check(self.lib.ifemgpu_learn_evaluate(self.ctx, C.byref(mse)))
        return mse.value

    def learn_gradients(self, X: np.ndarray, Y: np.ndarray):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        info = self.learn_info()
        assert X.shape[0] == Y.shape[0]
        assert X.shape[1] == info["inputs"] and Y.shape[1] == info["coarse_unknowns"]
        grad = np.zeros(info["nparam"], dtype=np.float32)
        loss = C.c_float()
        self._check(self.lib.ifemgpu_learn_gradients(self.ctx, _ptr(X), _ptr(Y), X.shape[0],
                                                     _ptr(grad), C.byref(loss)))
        return loss.value, grad

    def learn_get_weights(self):
        n = C.c_int()
        s = C.c_float()
        self._check(self.lib.ifemgpu_learn_get_weights(self.ctx, None, C.byref(n), C.byref(s)))
        theta = np.zeros(n.value, dtype=np.float32)
        self._check(self.lib.ifemgpu_learn_get_weights(self.ctx, _ptr(theta), C.byref(n),
                                                       C.byref(s)))
        return theta, s.value

    def learn_set_weights(self, theta: np.ndarray, scale: float):
        theta = np.ascontiguousarray(theta, dtype=np.float32)
        self._check(self.lib.ifemgpu_learn_set_weights(self.ctx, _ptr(theta), theta.size, scale))
