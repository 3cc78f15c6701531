"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the CPU FP64 oracle
(oracle/ifem_oracle.cpp), a restatement of IFEM's assembly path.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may use
this module, and only as the checker or the timed CPU baseline -- never as
part of the GPU product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ifem_oracle.cpp")
LIB = os.path.join(HERE, "libifem_oracle.so")


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (-O3, OpenMP)."""
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-shared", "-fPIC", SRC, "-o", LIB]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stderr}")
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P, I, D, V = C.c_void_p, C.c_int, C.c_double, C.c_void_p
        sig = {
            "ifo_create": (P, [I]), "ifo_destroy": (None, [P]),
            "ifo_set_bisect": (None, [P, I]),
            "ifo_add_patch": (I, [P, I, V, V, V, V, I]),
            "ifo_set_material": (I, [P, I, I, D, D, I, D, D, V]),
            "ifo_set_field": (I, [P, I, I, V]),
            "ifo_set_mass": (I, [P, I, D]),
            "ifo_connect": (I, [P, I, I, I, I, I]),
            "ifo_norms": (None, [P, V, V, V]),
            "ifo_secondary": (None, [P, I, V, V]),
            "ifo_constrain_face": (I, [P, I, I, I, D]),
            "ifo_add_neumann": (I, [P, I, I, V]),
            "ifo_preprocess": (I, [P, I]), "ifo_sizes": (None, [P, V]),
            "ifo_get_sam": (None, [P, V, V]), "ifo_get_pattern": (None, [P, V, V]),
            "ifo_get_mnpc": (I, [P, I, V]),
            "ifo_assemble": (C.c_long, [P, I, C.c_long]),
            "ifo_element": (I, [P, I, I, V, V]),
            "ifo_get_system": (None, [P, V, V]),
            "ifo_gauss": (None, [I, V, V]),
            "ifo_basis": (I, [P, I, V, V, V, V]),
            "ifo_jacobian": (D, [I, I, V, V, V, V]),
            "ifo_op_laplacian": (None, [I, I, V, D, D, V]),
            "ifo_op_elasticity": (None, [I, I, V, D, D, D, V]),
            "ifo_pcg": (I, [P, V, V, D, I, I, V]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class OracleModel:
    """Same model-input methods as ifem_gb300.ifemgpu.SIM."""

    def __init__(self, n_gauss: int = 4):
        self.L = lib()
        self.h = self.L.ifo_create(n_gauss)
        self._keep = []
        self.sizes = None

    def close(self):
        if self.h:
            self.L.ifo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_patch(self, patch) -> int:
        deg = np.ascontiguousarray(patch.degree, dtype=np.int32)
        nco = np.ascontiguousarray(patch.ncoef, dtype=np.int32)
        kn = [np.ascontiguousarray(k, dtype=np.float64) for k in patch.knots]
        karr = (C.c_void_p * 3)(*[_p(k) for k in kn] + [None] * (3 - patch.dim))
        coefs = np.ascontiguousarray(patch.coefs, dtype=np.float64)
        self._keep += [deg, nco, kn, coefs, karr]
        self._nel_all = getattr(self, "_nel_all", 0) + patch.nel
        return self.L.ifo_add_patch(self.h, patch.dim, _p(deg), _p(nco), C.cast(karr, C.c_void_p),
                                    _p(coefs), int(patch.rational))

    def set_material(self, pid, kind, kappa=1.0, source=0.0, source_shape=0, E=1.0, nu=0.3,
                     body=(0.0, 0.0, 0.0)):
        b = np.ascontiguousarray(body, dtype=np.float64)
        self.L.ifo_set_material(self.h, pid, kind, kappa, source, source_shape, E, nu, _p(b))

    def connect(self, master, mface, slave, sface, orient=0):
        self.L.ifo_connect(self.h, master, mface, slave, sface, orient)

    def set_mass(self, pid, scale):
        self.L.ifo_set_mass(self.h, pid, float(scale))

    def set_field(self, pid, which, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        self.L.ifo_set_field(self.h, pid, which, _p(v))

    def constrain_face(self, pid, face, dofs, value=0.0):
        self.L.ifo_constrain_face(self.h, pid, face, dofs, value)

    def add_neumann(self, pid, face, values):
        v = np.zeros(3)
        v[:len(values)] = values
        self.L.ifo_add_neumann(self.h, pid, face, _p(v))

    def preprocess(self, pattern: int = -1):
        """pattern: 0 IFEM's std::set couplings, 1 the parallel node-neighbour
        construction, -1 the latter only for large models (same arrays)."""
        self.L.ifo_preprocess(self.h, pattern)
        s = np.zeros(6, dtype=np.int32)
        self.L.ifo_sizes(self.h, _p(s))
        self.sizes = dict(nnod=int(s[0]), nel=int(s[1]), ndof=int(s[2]), neq=int(s[3]),
                          nceq=int(s[4]), nnz=int(s[5]))
        return self.sizes

    def sam(self):
        s = self.sizes
        madof = np.zeros(s["nnod"] + 1, dtype=np.int32)
        meqn = np.zeros(s["ndof"], dtype=np.int32)
        self.L.ifo_get_sam(self.h, _p(madof), _p(meqn))
        return madof, meqn

    def pattern(self):
        s = self.sizes
        IA = np.zeros(s["neq"] + 1, dtype=np.int32)
        JA = np.zeros(max(s["nnz"], 1), dtype=np.int32)
        self.L.ifo_get_pattern(self.h, _p(IA), _p(JA))
        return IA, JA[:s["nnz"]]

    def mnpc(self, pid, nel, nen):
        out = np.zeros(nel * nen, dtype=np.int32)
        self.L.ifo_get_mnpc(self.h, pid, _p(out))
        return out.reshape(nel, nen)

    def set_bisect(self, on: bool = True):
        """Entry lookup of the scatter by binary search instead of IFEM's
        linear std::find (same sums; for parity tests of large models)."""
        self.L.ifo_set_bisect(self.h, int(on))

    def assemble(self, threads: int = 1, max_elements: int = 0) -> int:
        return self.L.ifo_assemble(self.h, threads, max_elements)

    def system(self):
        s = self.sizes
        A = np.zeros(s["nnz"])
        b = np.zeros(s["neq"])
        self.L.ifo_get_system(self.h, _p(A), _p(b))
        return A, b

    def element(self, pid, iel, nd):
        eK = np.zeros(nd * nd)
        eS = np.zeros(nd)
        n = self.L.ifo_element(self.h, pid, iel, _p(eK), _p(eS))
        return eK.reshape(nd, nd).T.copy(), eS, n  # row-major eK[i, j]

    def norms(self, u_dof, per_element=False):
        u = np.ascontiguousarray(u_dof, dtype=np.float64)
        tot = np.zeros(2)
        el = np.zeros((self._nel_all, 2)) if per_element else None
        self.L.ifo_norms(self.h, _p(u), _p(tot), _p(el) if per_element else None)
        return (tot, el) if per_element else tot

    def secondary(self, pid, u_dof, nel, nq, ncomp):
        u = np.ascontiguousarray(u_dof, dtype=np.float64)
        out = np.zeros((nel, nq, ncomp))
        self.L.ifo_secondary(self.h, pid, _p(u), _p(out))
        return out

    def pcg(self, b, rtol=1e-10, maxit=100000, threads=1, x0=None):
        x = np.zeros(self.sizes["neq"]) if x0 is None else np.array(x0, dtype=np.float64)
        rel = np.zeros(1)
        b = np.ascontiguousarray(b, dtype=np.float64)
        it = self.L.ifo_pcg(self.h, _p(b), _p(x), rtol, maxit, threads, _p(rel))
        return x, it, float(rel[0])


def gauss(n: int):
    x = np.zeros(n)
    w = np.zeros(n)
    lib().ifo_gauss(n, _p(x), _p(w))
    return x, w


def jacobian(dim, Xn, dNdu):
    """Xn: nen x dim, dNdu: nen x dim -> (det, J (dim x dim), dNdX nen x dim)."""
    nen = Xn.shape[0]
    Xc = np.ascontiguousarray(Xn, dtype=np.float64)
    dn = np.ascontiguousarray(np.asarray(dNdu, dtype=np.float64).T)   # column-major nen x dim
    J = np.zeros(dim * dim)
    dX = np.zeros(nen * dim)
    det = lib().ifo_jacobian(dim, nen, _p(Xc), _p(dn), _p(J), _p(dX))
    return det, J.reshape(dim, dim).T, dX.reshape(dim, nen).T


def op_laplacian(dNdX, kappa=1.0, detJxW=1.0):
    nen, dim = dNdX.shape
    d = np.ascontiguousarray(np.asarray(dNdX, dtype=np.float64).T)
    eK = np.zeros(nen * nen)
    lib().ifo_op_laplacian(dim, nen, _p(d), kappa, detJxW, _p(eK))
    return eK.reshape(nen, nen).T


def op_elasticity(dNdX, lam, mu, detJxW=1.0):
    nen, dim = dNdX.shape
    d = np.ascontiguousarray(np.asarray(dNdX, dtype=np.float64).T)
    nd = nen * dim
    eK = np.zeros(nd * nd)
    lib().ifo_op_elasticity(dim, nen, _p(d), lam, mu, detJxW, _p(eK))
    return eK.reshape(nd, nd).T
