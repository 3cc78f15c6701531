"""TEST INFRASTRUCTURE ONLY: one spline patch assembled by IFEM's own code.

oracle/_ref/libifem_ref.so (built from the IFEM sources by
oracle/ref/build_ref.py, only where those sources are present) holds IFEM's
SAMpatch numbering, SparseMatrix pattern (SuperLU layout), utl::Jacobian,
EqualOrderOperators::Weak::Laplacian/Source and SAM::assembleSystem, driven by
oracle/ref/ref_harness.cpp.  This module feeds it a patch:

* MNPC and the fixed DOFs come from the CPU oracle (its restatement of
  ASMs3D::generateFEMTopology/createMNPC/constrainFace, which need GoTools);
* basis values at IFEM's Gauss points (GaussQuadrature tables, taken from the
  compiled reference) come from the oracle's spline evaluation, the part that
  IFEM delegates to GoTools;
* Poisson element matrices and load vectors are formed by IFEM's operators;
  elasticity element matrices (IFEM's elasticity integrand lives outside the
  IFEM tree) come from the oracle and are scattered by IFEM's SAM.

Used to pin the oracle's global system, and to write the golden systems under
tests/golden/ that the GPU tests compare against.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libifem_ref.so")

_lib = None


def available() -> bool:
    return os.path.exists(LIB)


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(LIB)
        P, I, V = C.c_void_p, C.c_int, C.c_void_p
        sig = {
            "rh_create": (P, [I, I, I, I, I, V]), "rh_destroy": (None, [P]),
            "rh_fix": (I, [P, I, I]), "rh_init": (I, [P, V]),
            "rh_gauss": (None, [I, V, V]),
            "rh_poisson_element": (I, [P, I, I, V, V, V, V, V, C.c_double, V, V, V]),
            "rh_assemble": (I, [P, I, V, V]),
            "rh_get_sam": (None, [P, V, V]), "rh_get_system": (None, [P, V, V, V, V]),
            "rh_dump": (I, [P, C.c_char_p, C.c_char_p, I, C.c_double]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def gauss(n: int):
    """IFEM's Gauss rule of n points (src/Utility/GaussQuadrature.C tables)."""
    x, w = np.zeros(n), np.zeros(n)
    lib().rh_gauss(n, _p(x), _p(w))
    return x, w


def reference_system(patch, n_gauss: int, dumps=None, zero_tol: float = 0.0):
    """K (CSC: IA, JA, A), b, MADOF, MEQN of one patch from IFEM's code.

    n_gauss follows ASMbase::getNoGaussPt: 1..10 points, 0 for p+1 per
    direction.  b is returned for Poisson patches only (elasticity tractions
    are integrated on faces, outside this harness).  dumps: optional list of
    (format, matrix_path, rhs_path) written by IFEM's SparseMatrix::dump and
    StdVector::dump (LinAlg::StorageFormat numbers)."""
    import oracle
    from ifem_gb300 import workloads as W

    orc = oracle.OracleModel(n_gauss)
    W.load_into(orc, [patch])
    orc.preprocess()
    madof_o, meqn_o = orc.sam()
    dim, p = patch.dim, patch.degree
    nen = int(np.prod([q + 1 for q in p]))
    nel = patch.nel
    nf = 1 if patch.kind == 1 else dim
    mnpc = orc.mnpc(1, nel, nen).astype(np.int32)
    L = lib()
    h = L.rh_create(dim, nf, patch.nnod, nel, nen, _p(np.ascontiguousarray(mnpc)))
    try:
        for n in range(patch.nnod):
            code = 0
            for d in range(nf):
                if meqn_o[madof_o[n] - 1 + d] == 0:
                    code = 10 * code + d + 1
            if code:
                L.rh_fix(h, n + 1, code)
        s = np.zeros(4, dtype=np.int32)
        if L.rh_init(h, _p(s)) != 0:
            raise RuntimeError("SAMpatch::init failed")
        nnod, ndof, neq, nnz = (int(v) for v in s)
        if patch.kind == 1:
            _poisson_elements(L, h, orc, patch, n_gauss, mnpc, nen)
        else:
            nd = nf * nen
            for e in range(nel):
                eK, eS, _ = orc.element(1, e, nd)    # 0-based element index
                if L.rh_assemble(h, e + 1, _p(np.ascontiguousarray(eK.ravel(order="F"))),
                                 _p(np.ascontiguousarray(eS))) != 0:
                    raise RuntimeError("SAM::assembleSystem failed")
        IA = np.zeros(neq + 1, dtype=np.int32)
        JA = np.zeros(nnz, dtype=np.int32)
        A = np.zeros(nnz)
        b = np.zeros(neq)
        L.rh_get_system(h, _p(IA), _p(JA), _p(A), _p(b))
        madof = np.zeros(nnod + 1, dtype=np.int32)
        meqn = np.zeros(ndof, dtype=np.int32)
        L.rh_get_sam(h, _p(madof), _p(meqn))
        for fmt, mpath, rpath in dumps or ():
            L.rh_dump(h, mpath.encode() if mpath else None, rpath.encode() if rpath else None,
                      fmt, zero_tol)
    finally:
        L.rh_destroy(h)
        orc.close()
    return dict(IA=IA, JA=JA, A=A, b=b if patch.kind == 1 else None, madof=madof, meqn=meqn)


def _poisson_elements(L, h, orc, patch, n_gauss, mnpc, nen):
    """The element loop of ASMs3D/ASMs2D::integrate with IFEM's operators."""
    dim, p = patch.dim, patch.degree
    ng = [n_gauss if n_gauss > 0 else p[d] + 1 for d in range(dim)]
    rules = [gauss(n) for n in ng]
    nel_d = [patch.ncoef[d] - p[d] for d in range(dim)]
    X = np.zeros((patch.nnod, 3))
    X[:, :dim] = patch.coefs[:, :dim]
    logk = None if patch.log_kappa is None else np.asarray(patch.log_kappa)
    noise = None if patch.noise is None else np.asarray(patch.noise)
    nq = int(np.prod(ng))
    Nq = np.zeros((nq, nen))
    dNq = np.zeros((nq, dim, nen))
    wfac = np.zeros(nq)
    kap = np.zeros(nq)
    f = np.zeros(nq)
    eK = np.zeros(nen * nen)
    eS = np.zeros(nen)
    u = np.zeros(3)
    Nb = np.zeros(nen)
    dNb = np.zeros(nen * dim)
    nodes = np.zeros(nen, dtype=np.int32)
    for e in range(patch.nel):
        idx, r = [], e
        for d in range(dim):
            idx.append(r % nel_d[d])
            r //= nel_d[d]
        spans = [(patch.knots[d][p[d] + idx[d]], patch.knots[d][p[d] + idx[d] + 1])
                 for d in range(dim)]
        dV = np.prod([0.5 * (b1 - b0) for b0, b1 in spans])
        q = 0
        for gk in range(ng[2] if dim == 3 else 1):
            for gj in range(ng[1]):
                for gi in range(ng[0]):
                    g = (gi, gj, gk)
                    w = dV
                    for d in range(dim):
                        xi, wt = rules[d]
                        b0, b1 = spans[d]
                        u[d] = 0.5 * ((b1 - b0) * xi[g[d]] + b1 + b0)
                        w *= wt[g[d]]
                    orc.L.ifo_basis(orc.h, 1, _p(u), _p(Nb), _p(dNb), _p(nodes))
                    if not np.array_equal(nodes, mnpc[e]):
                        raise RuntimeError("basis node order differs from MNPC")
                    Nq[q] = Nb
                    dNq[q] = dNb.reshape(dim, nen)
                    wfac[q] = w
                    k = patch.kappa
                    if logk is not None:
                        k *= np.exp(Nb @ logk[mnpc[e]])
                    kap[q] = k
                    src = patch.source
                    if src != 0.0:
                        xq = Nb @ X[mnpc[e]]
                        if patch.source_shape == 1:
                            src *= np.prod(np.sin(np.pi * xq[:dim]))
                        if noise is not None:
                            src *= 1.0 + Nb @ noise[mnpc[e]]
                    f[q] = src
                    q += 1
        Xe = np.ascontiguousarray(X[mnpc[e]])
        L.rh_poisson_element(h, e + 1, nq, _p(np.ascontiguousarray(Nq)),
                             _p(np.ascontiguousarray(dNq)), _p(wfac), _p(kap), _p(f),
                             float(patch.mass), _p(Xe), _p(eK), _p(eS))
