"""The oracle's solution norms and secondary solution against closed forms:
constant and linear fields on a box, rigid motion and uniaxial strain in
elasticity (test infrastructure for the GPU norms kernel)."""
import numpy as np

from ifem_gb300 import workloads as W


def model(pc, ng=3):
    import oracle
    o = oracle.OracleModel(ng)
    W.load_into(o, [pc])
    o.preprocess()
    return o


def test_poisson_constant_and_linear_fields(oracle_lib):
    pc = W.box_patch(3, 2, 4, size=(1.0, 2.0, 0.5))
    pc.kind = 1
    o = model(pc)
    nd = o.sizes["ndof"]
    e, l2 = o.norms(np.ones(nd))
    assert abs(e) < 1e-12 and abs(l2 - 1.0) < 1e-12
    e, l2 = o.norms(pc.coefs[:, 0])            # u = x reproduced exactly by p=2
    assert abs(e - 1.0) < 1e-12 and abs(l2 - 1.0 / 3.0) < 1e-12
    flux = o.secondary(1, pc.coefs[:, 0], pc.nel, 27, 3)
    assert np.abs(flux[..., 0] + 1.0).max() < 1e-12 and np.abs(flux[..., 1:]).max() < 1e-12


def test_elasticity_rigid_motion_and_uniaxial_strain(oracle_lib):
    pe = W.perturb(W.box_patch(3, 2, 3), np.random.default_rng(7), 0.05, weights=(1.0, 1.0))
    pe.kind = 2
    o = model(pe)
    e, _ = o.norms(np.tile([0.3, -0.2, 0.1], pe.nnod))
    assert abs(e) < 1e-12
    u = np.zeros(3 * pe.nnod)
    u[0::3] = pe.coefs[:, 0]                   # u_x = x: eps_xx = 1
    lam, mu = 0.3 / (1.3 * 0.4), 1.0 / 2.6
    vol = o.norms(np.tile([1.0, 0.0, 0.0], pe.nnod))[1]   # int 1 dV
    e, _ = o.norms(u)
    assert abs(e - (lam + 2 * mu) * vol) < 1e-10 * vol
    s = o.secondary(1, u, pe.nel, 27, 6)
    assert np.abs(s[..., 0] - (lam + 2 * mu)).max() < 1e-10
    assert np.abs(s[..., 1:3] - lam).max() < 1e-10 and np.abs(s[..., 3:]).max() < 1e-10
