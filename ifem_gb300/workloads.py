"""Seeded synthetic spline models for the five benchmark configurations.

No public dataset is involved: every model is generated here from
``numpy.random.default_rng(seed)``, default seed 20261203 + configuration
number, and fed unchanged to the GPU path and to the CPU oracle.

  config 1  2D Poisson, p=2, 32x32 elements, 3x3 Gauss, f = sin(pi x) sin(pi y)
            (1 + sum_a R_a eta_a), eta_a ~ 0.1 N(0,1); u = 0 on all edges.
  config 2  3D linear elasticity on one NURBS patch, p=2, 24^3 elements,
            3x3x3 Gauss, E=1, nu=0.3, Greville control points perturbed by
            U(-0.1h, 0.1h), weights U[0.8, 1.2]; clamped on w=0 (face 5),
            unit traction (0,0,1) on w=1 (face 6).
  config 3  64 independent patches offset in space, n_e ~ U{8..32} per
            direction, p ~ U{2,3}, Poisson or elasticity; geometry as config 2.
  config 4  3D Poisson, p=3, 64^3 elements, 4x4x4 Gauss, kappa = exp(sum_a R_a
            g_a) with g a Gaussian random field (sigma 1, squared-exponential
            correlation length 0.1) on the control net; f = 1, u = 0 on all faces.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

BASE_SEED = 20261203


@dataclass
class SplinePatch:
    dim: int
    degree: tuple
    ncoef: tuple
    knots: list
    coefs: np.ndarray          # nnod x (dim [+1 weight])
    rational: bool = False
    # physics attached to the patch
    kind: int = 1              # 1 Poisson, 2 elasticity
    kappa: float = 1.0
    source: float = 0.0
    source_shape: int = 0
    E: float = 1.0
    nu: float = 0.3
    body: tuple = (0.0, 0.0, 0.0)
    mass: float = 0.0          # scale of the consistent mass matrix added to K
    log_kappa: np.ndarray | None = None
    noise: np.ndarray | None = None
    dirichlet: list = field(default_factory=list)   # (face, dofs, value)
    neumann: list = field(default_factory=list)     # (face, values)

    @property
    def nnod(self) -> int:
        return int(np.prod(self.ncoef))

    @property
    def nel(self) -> int:
        return int(np.prod([n - p for n, p in zip(self.ncoef, self.degree)]))


def uniform_knots(p: int, nel: int) -> np.ndarray:
    inner = np.arange(1, nel) / nel
    return np.concatenate([np.zeros(p + 1), inner, np.ones(p + 1)])


def greville(knots: np.ndarray, p: int) -> np.ndarray:
    n = len(knots) - p - 1
    return np.array([knots[i + 1:i + p + 1].mean() for i in range(n)])


def box_patch(dim: int, p, nel, origin=(0.0, 0.0, 0.0), size=(1.0, 1.0, 1.0)) -> SplinePatch:
    """Identity-map patch over a box: control points at the Greville abscissae."""
    p = tuple(int(x) for x in (p if np.ndim(p) else [p] * dim))
    nel = tuple(int(x) for x in (nel if np.ndim(nel) else [nel] * dim))
    knots = [uniform_knots(p[d], nel[d]) for d in range(dim)]
    g = [origin[d] + size[d] * greville(knots[d], p[d]) for d in range(dim)]
    mesh = np.meshgrid(*g, indexing="ij")            # axis 0 = first index
    # node-major with the first index fastest
    coefs = np.stack([m.transpose(tuple(range(dim))[::-1]).ravel() for m in mesh], axis=1)
    ncoef = tuple(len(x) for x in g)
    return SplinePatch(dim, p, ncoef, knots, coefs)


def perturb(patch: SplinePatch, rng, amp: float, weights=(0.8, 1.2)) -> SplinePatch:
    """Control points += U(-amp*h, amp*h), h the smallest element size; rational
    weights U[weights]."""
    h = min(1.0 / (n - p) for n, p in zip(patch.ncoef, patch.degree))
    xyz = patch.coefs[:, :patch.dim] + rng.uniform(-amp * h, amp * h, size=(patch.nnod, patch.dim))
    w = rng.uniform(weights[0], weights[1], size=(patch.nnod, 1))
    patch.coefs = np.concatenate([xyz, w], axis=1)
    patch.rational = True
    return patch


def gaussian_field_3d(rng, points: np.ndarray, sigma: float = 1.0, corr: float = 0.1,
                      grid: int = 64) -> np.ndarray:
    """Zero-mean Gaussian random field with covariance sigma^2 exp(-r^2/(2 corr^2)),
    sampled on a uniform grid over [0,1]^3 by circulant embedding (FFT on the
    doubled periodic grid, negative eigenvalues clipped) and interpolated
    trilinearly to `points` (n x 3)."""
    m = 2 * grid
    h = 1.0 / (grid - 1)
    k = np.arange(m)
    d = np.minimum(k, m - k) * h
    r2 = d[:, None, None] ** 2 + d[None, :, None] ** 2 + d[None, None, :] ** 2
    c = sigma ** 2 * np.exp(-r2 / (2 * corr ** 2))
    lam = np.fft.fftn(c).real
    lam = np.maximum(lam, 0.0)
    xi = rng.standard_normal((m, m, m)) + 1j * rng.standard_normal((m, m, m))
    f = np.fft.fftn(np.sqrt(lam / m ** 3) * xi)
    g = f.real[:grid, :grid, :grid]
    # trilinear interpolation
    t = np.clip(points / h, 0, grid - 1 - 1e-9)
    i0 = np.floor(t).astype(int)
    w = t - i0
    out = np.zeros(len(points))
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                wt = ((w[:, 0] if dx else 1 - w[:, 0]) * (w[:, 1] if dy else 1 - w[:, 1]) *
                      (w[:, 2] if dz else 1 - w[:, 2]))
                out += wt * g[i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz]
    return out


# ---- configurations ---------------------------------------------------------

def config1(nel: int = 32, p: int = 2, seed: int | None = None) -> tuple[list, int]:
    rng = np.random.default_rng(BASE_SEED + 1 if seed is None else seed)
    pc = box_patch(2, p, nel)
    pc.kind = 1
    pc.source = 1.0
    pc.source_shape = 1
    pc.noise = 0.1 * rng.standard_normal(pc.nnod)
    pc.dirichlet = [(f, 1, 0.0) for f in (1, 2, 3, 4)]
    return [pc], 3


def config2(nel: int = 24, p: int = 2, seed: int | None = None) -> tuple[list, int]:
    rng = np.random.default_rng(BASE_SEED + 2 if seed is None else seed)
    pc = perturb(box_patch(3, p, nel), rng, 0.1)
    pc.kind = 2
    pc.E, pc.nu = 1.0, 0.3
    pc.dirichlet = [(5, 123, 0.0)]
    pc.neumann = [(6, (0.0, 0.0, 1.0))]
    return [pc], 3


def config3(npatch: int = 64, seed: int | None = None, nmin: int = 8, nmax: int = 32):
    rng = np.random.default_rng(BASE_SEED + 3 if seed is None else seed)
    patches = []
    for i in range(npatch):
        ne = int(rng.integers(nmin, nmax + 1))
        p = int(rng.integers(2, 4))
        kind = int(rng.integers(1, 3))
        origin = (2.0 * (i % 4), 2.0 * ((i // 4) % 4), 2.0 * (i // 16))
        pc = perturb(box_patch(3, p, ne, origin=origin), rng, 0.1)
        pc.kind = kind
        if kind == 1:
            pc.source = 1.0
            pc.dirichlet = [(f, 1, 0.0) for f in range(1, 7)]
        else:
            pc.dirichlet = [(5, 123, 0.0)]
            pc.neumann = [(6, (0.0, 0.0, 1.0))]
        patches.append(pc)
    return patches, 0    # nGauss = 0: degree+1 points per patch (IFEM convention)


def config4(nel: int = 64, p: int = 3, seed: int | None = None, grid: int = 64):
    rng = np.random.default_rng(BASE_SEED + 4 if seed is None else seed)
    pc = box_patch(3, p, nel)
    pc.kind = 1
    pc.source = 1.0
    pc.log_kappa = gaussian_field_3d(rng, pc.coefs[:, :3], grid=grid)
    pc.dirichlet = [(f, 1, 0.0) for f in range(1, 7)]
    return [pc], 4


def connected_boxes(kind: int = 1, p: int = 2, nel: int = 3, npatch: int = 2,
                    rotated: bool = False):
    """npatch unit cubes of nel^3 elements along x, conformingly connected
    (patch i's +x face is patch i+1's -x face).  With rotated, the even
    patches are parameterised (i, j, k) -> (x, z, 1 - y), so that the
    connections onto them need face orientation 5 and those from them 6
    (swapped and reversed parameter directions).  Poisson (kind 1: conductivity 1 + patch index, unit
    source, u = 0 on the outer x faces) or elasticity (kind 2: clamped -x face
    of the first patch, unit traction on the +x face of the last).
    Returns (patches, n_gauss, connections)."""
    patches, conns = [], []
    for ip in range(npatch):
        pc = box_patch(3, p, nel, origin=(float(ip), 0.0, 0.0))
        if rotated and ip % 2 == 1:
            g = greville(uniform_knots(p, nel), p)
            n = len(g)
            i, j, k = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
            order = lambda a: a.transpose(2, 1, 0).ravel()   # first index fastest
            pc.coefs = np.stack([ip + g[order(i)], 1.0 - g[order(k)], g[order(j)]], axis=1)
        pc.kind = kind
        patches.append(pc)
        if ip > 0:  # orientation 5 onto a rotated patch, 6 from one, else 0
            orient = 0 if not rotated else (5 if ip % 2 == 1 else 6)
            conns.append((ip, 2, ip + 1, 1, orient))
    if kind == 1:
        for ip, pc in enumerate(patches):
            pc.kappa = 1.0 + ip
            pc.source = 1.0
        patches[0].dirichlet = [(1, 1, 0.0)]
        patches[-1].dirichlet = [(2, 1, 0.0)]
    else:
        patches[0].dirichlet = [(1, 123, 0.0)]
        patches[-1].neumann = [(2, (1.0, 0.0, 0.0))]
    return patches, 3, conns


def load_into(sim, patches, connections=()) -> list[int]:
    """Feed patches to an ifem_gb300.ifemgpu.SIM (or the oracle wrapper);
    connections: (master, mface, slave, sface, orient) tuples, 1-based."""
    ids = []
    for pc in patches:
        pid = sim.add_patch(pc)
        sim.set_material(pid, pc.kind, kappa=pc.kappa, source=pc.source,
                         source_shape=pc.source_shape, E=pc.E, nu=pc.nu, body=pc.body)
        if pc.mass:
            sim.set_mass(pid, pc.mass)
        if pc.log_kappa is not None:
            sim.set_field(pid, 1, pc.log_kappa)
        if pc.noise is not None:
            sim.set_field(pid, 2, pc.noise)
        for face, dofs, value in pc.dirichlet:
            sim.constrain_face(pid, face, dofs, value)
        for face, vals in pc.neumann:
            sim.add_neumann(pid, face, vals)
        ids.append(pid)
    for c in connections:
        sim.connect(*c)
    return ids
