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
            "rh_create_multi": (P, [I, I, I, V, V, I, V]),
            "rh_collapse": (I, [P, I, I, I, I]), "rh_neighbours": (None, [P, I, I]),
            "rh_renumber": (I, [P]), "rh_fix_patch": (I, [P, I, I, I]),
            "rh_node_id": (I, [P, I, I]), "rh_elm_id": (I, [P, I, I]),
            "rh_secondary_points": (I, [I, I, I, V, V, V, I, V, V, C.c_double, C.c_double, V]),
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


def face_nodes(patch, face):
    """0-based patch nodes of a face (3D) or edge (2D) in IFEM's order
    (ASMs3D::getBoundaryNodes, src/ASM/ASMs3D.C:1770-1818)."""
    n1, n2 = patch.ncoef[0], patch.ncoef[1]
    n3 = patch.ncoef[2] if patch.dim == 3 else 1
    d, hi = (face + 1) // 2, face % 2 == 0
    idx = lambda i, j, k: (k * n2 + j) * n1 + i
    if d == 1:
        return [idx(n1 - 1 if hi else 0, j, k) for k in range(n3) for j in range(n2)]
    if d == 2:
        return [idx(i, n2 - 1 if hi else 0, k) for k in range(n3) for i in range(n1)]
    return [idx(i, j, n3 - 1 if hi else 0) for j in range(n2) for i in range(n1)]


def face_size(patch, face):
    """ASMs3D::getFaceSize (src/ASM/ASMs3D.C:3796-3810); 2D: (edge nodes, 1)."""
    n = list(patch.ncoef) + [1] * (3 - patch.dim)
    d = (face + 1) // 2
    if patch.dim == 2:
        return (n[1] if d == 1 else n[0]), 1
    return {1: (n[1], n[2]), 2: (n[0], n[2]), 3: (n[0], n[1])}[d]


def connection_pairs(pm, mface, ps, sface, orient):
    """(master node, slave node) pairs, 0-based, in the loop order of
    ASMs3D::connectBasis / ASMs2D::connectBasis."""
    mn, sn = face_nodes(pm, mface), face_nodes(ps, sface)
    m1, m2 = face_size(ps, sface)
    n1, n2 = face_size(pm, mface)
    pairs, node = [], 0
    for j in range(n2):
        for i in range(n1):
            if pm.dim == 3:
                k, l = {0: (i, j), 1: (i, n2 - j - 1), 2: (n1 - i - 1, j), 3: (n1 - i - 1, n2 - j - 1),
                        4: (j, i), 5: (j, m2 - i - 1), 6: (m1 - j - 1, i),
                        7: (m1 - j - 1, m2 - i - 1)}[orient]
            else:
                k, l = (n1 - i - 1 if orient else i), 0
            pairs.append((mn[node], sn[l * m1 + k]))
            node += 1
    return pairs


def reference_system_multi(patches, connections, n_gauss: int):
    """As reference_system for a model of several patches joined by
    conforming connections (master, mface, slave, sface, orient): IFEM's
    ASMbase::collapseNodes over the node pairs of each connection, its
    neighbour registration, SIMbase::renumberNodes, SAMpatch::init over all
    patches and SAM::assembleSystem with global element numbers.  Homogeneous
    Dirichlet faces only."""
    import oracle
    from ifem_gb300 import workloads as W

    orc = oracle.OracleModel(n_gauss)
    W.load_into(orc, patches, connections)
    orc.preprocess()
    dim = patches[0].dim
    nen = int(np.prod([q + 1 for q in patches[0].degree]))
    nf = 1 if patches[0].kind == 1 else dim
    mnpcs = [orc.mnpc(i + 1, pc.nel, nen).astype(np.int32) for i, pc in enumerate(patches)]
    L = lib()
    nn = np.array([pc.nnod for pc in patches], dtype=np.int32)
    ne = np.array([pc.nel for pc in patches], dtype=np.int32)
    allm = np.ascontiguousarray(np.concatenate([m.ravel() for m in mnpcs]))
    h = L.rh_create_multi(dim, nf, len(patches), _p(nn), _p(ne), nen, _p(allm))
    try:
        for (m, mf, s, sf, o) in connections:
            for a, b in connection_pairs(patches[m - 1], mf, patches[s - 1], sf, o):
                L.rh_collapse(h, m, a + 1, s, b + 1)
            L.rh_neighbours(h, m, s)
        L.rh_renumber(h)
        for i, pc in enumerate(patches):
            for face, dofs, value in pc.dirichlet:
                if value != 0.0:
                    raise ValueError("homogeneous Dirichlet conditions only")
                for node in face_nodes(pc, face):
                    L.rh_fix_patch(h, i + 1, node + 1, dofs)
        s = np.zeros(4, dtype=np.int32)
        if L.rh_init(h, _p(s)) != 0:
            raise RuntimeError("SAMpatch::init failed")
        nnod, ndof, neq, nnz = (int(v) for v in s)
        for i, pc in enumerate(patches):
            iel = [L.rh_elm_id(h, i + 1, e) for e in range(pc.nel)]
            if pc.kind == 1:
                _poisson_elements(L, h, orc, pc, n_gauss, mnpcs[i], nen, pid=i + 1, iel=iel)
            else:
                nd = nf * nen
                for e in range(pc.nel):
                    eK, eS, _ = orc.element(i + 1, e, nd)
                    if L.rh_assemble(h, iel[e], _p(np.ascontiguousarray(eK.ravel(order="F"))),
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
    finally:
        L.rh_destroy(h)
        orc.close()
    return dict(IA=IA, JA=JA, A=A, b=b if patches[0].kind == 1 else None, madof=madof,
                meqn=meqn)


def _poisson_elements(L, h, orc, patch, n_gauss, mnpc, nen, pid=1, iel=None):
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
                    orc.L.ifo_basis(orc.h, pid, _p(u), _p(Nb), _p(dNb), _p(nodes))
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
        L.rh_poisson_element(h, iel[e] if iel else e + 1, nq, _p(np.ascontiguousarray(Nq)),
                             _p(np.ascontiguousarray(dNq)), _p(wfac), _p(kap), _p(f),
                             float(patch.mass), _p(Xe), _p(eK), _p(eS))


def reference_secondary(patch, n_gauss: int, u_dof):
    """Secondary solution of u (DOF order, npv values per node) at every Gauss
    point of one patch with IFEM's utl::Jacobian: Poisson flux -kappa grad u,
    elasticity stress (Voigt xx yy zz xy yz zx).  Shape (nel, nq, ncomp),
    elements and points first index fastest.  Basis values at IFEM's Gauss
    points come from the oracle (IFEM takes them from GoTools)."""
    import oracle
    from ifem_gb300 import workloads as W

    orc = oracle.OracleModel(n_gauss)
    W.load_into(orc, [patch])
    orc.preprocess()
    dim, p = patch.dim, patch.degree
    nen = int(np.prod([q + 1 for q in p]))
    nf = 1 if patch.kind == 1 else dim
    ncomp = dim if nf == 1 else 6
    mnpc = orc.mnpc(1, patch.nel, nen)
    ng = [n_gauss if n_gauss > 0 else p[d] + 1 for d in range(dim)]
    rules = [gauss(n) for n in ng]
    nel_d = [patch.ncoef[d] - p[d] for d in range(dim)]
    X = np.zeros((patch.nnod, 3))
    X[:, :dim] = patch.coefs[:, :dim]
    logk = None if patch.log_kappa is None else np.asarray(patch.log_kappa)
    lam = patch.E * patch.nu / ((1 + patch.nu) * (1 - 2 * patch.nu))
    mu = patch.E / (2 * (1 + patch.nu))
    u_dof = np.asarray(u_dof, dtype=np.float64).reshape(patch.nnod, nf)
    nq = int(np.prod(ng))
    out = np.zeros((patch.nel, nq, ncomp))
    Nq = np.zeros((nq, nen))
    dNq = np.zeros((nq, dim, nen))
    kap = np.zeros(nq)
    u = np.zeros(3)
    Nb = np.zeros(nen)
    dNb = np.zeros(nen * dim)
    nodes = np.zeros(nen, dtype=np.int32)
    L = lib()
    try:
        for e in range(patch.nel):
            idx, r = [], e
            for d in range(dim):
                idx.append(r % nel_d[d])
                r //= nel_d[d]
            spans = [(patch.knots[d][p[d] + idx[d]], patch.knots[d][p[d] + idx[d] + 1])
                     for d in range(dim)]
            q = 0
            for gk in range(ng[2] if dim == 3 else 1):
                for gj in range(ng[1]):
                    for gi in range(ng[0]):
                        g = (gi, gj, gk)
                        for d in range(dim):
                            xi, _ = rules[d]
                            b0, b1 = spans[d]
                            u[d] = 0.5 * ((b1 - b0) * xi[g[d]] + b1 + b0)
                        orc.L.ifo_basis(orc.h, 1, _p(u), _p(Nb), _p(dNb), _p(nodes))
                        Nq[q] = Nb
                        dNq[q] = dNb.reshape(dim, nen)
                        k = patch.kappa
                        if logk is not None:
                            k *= np.exp(Nb @ logk[mnpc[e]])
                        kap[q] = k
                        q += 1
            ue = np.ascontiguousarray(u_dof[mnpc[e]].ravel())
            res = np.zeros((nq, ncomp))
            L.rh_secondary_points(dim, nen, nq, _p(np.ascontiguousarray(Nq)),
                                  _p(np.ascontiguousarray(dNq)),
                                  _p(np.ascontiguousarray(X[mnpc[e]])), nf, _p(ue), _p(kap),
                                  lam, mu, _p(res))
            out[e] = res
    finally:
        orc.close()
    return out
