"""SUPG advection-diffusion (the reference's AdvectionDiffusion, method "SUPG").

CPU: the oracle restatement relaxes pure diffusion between Dirichlet walls to
the linear profile and its time-step bound follows the reference's formula.
GPU: uwg_advdiff_step and uwg_advdiff_max_dt through the C ABI against the
oracle, 1e-12 relative over several steps in 2D and 3D, and the uw-style
``AdvectionDiffusion`` against the same oracle.
"""
import numpy as np
import pytest
import torch

import oracle
from oracle import advdiff


def _walls(m, axis):
    nodes = m.node_coords()
    return np.isclose(nodes[:, axis], 0.0) | np.isclose(nodes[:, axis], 1.0)


def test_oracle_pure_diffusion_steady_state():
    m = oracle.Mesh(2, 1, (6, 6), (0.0, 0.0), (1.0, 1.0))
    nodes = m.node_coords()
    bc = _walls(m, 1)
    bcval = np.where(np.isclose(nodes[:, 1], 0.0), 1.0, 0.0)
    phi = np.zeros(m.n_nodes)
    phidot = np.zeros(m.n_nodes)
    kappa = np.ones((m.n_el, 9))
    dt = advdiff.max_dt(m, None, kappa)
    assert dt == pytest.approx(0.5 * (1.0 / 6) ** 2)
    for _ in range(400):
        phi, phidot = advdiff.step(m, dt, None, kappa, None, bc, bcval, None, phi, phidot)
    assert np.abs(phi - (1.0 - nodes[:, 1])).max() < 1e-5


def _case(dim, res, seed):
    rng = np.random.default_rng(seed)
    m = oracle.Mesh(dim, 1, res, (0.0,) * dim, (1.0,) * dim)
    nodes = m.node_coords()
    vel = rng.uniform(-1.0, 1.0, (m.n_nodes, dim))
    vel[:, dim - 1] += 0.5
    nq = 3 ** dim
    kappa = rng.uniform(1e-3, 2e-2, (m.n_el, nq))
    src = rng.uniform(-0.1, 0.1, (m.n_el, nq))
    bc = _walls(m, dim - 1)
    bcval = np.where(np.isclose(nodes[:, dim - 1], 0.0), 1.0, 0.0)
    phi = rng.uniform(0.0, 1.0, m.n_nodes)
    phidot = rng.uniform(-0.1, 0.1, m.n_nodes)
    return m, vel, kappa, src, bc, bcval, phi, phidot


@pytest.mark.gpu
@pytest.mark.parametrize("dim,res", [(2, (8, 6)), (3, (4, 3, 3))])
def test_supg_step_matches_oracle(gpu, dim, res):
    from underworld2_gb300._core import Context
    m, vel, kappa, src, bc, bcval, phi, phidot = _case(dim, res, 5)
    c = Context(dim, res, (0.0,) * dim, (1.0,) * dim)
    t = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    vel_t, kap_t, src_t = t(vel.ravel()), t(kappa.ravel()), t(src.ravel())
    phi_t, pd_t, bcv_t = t(phi), t(phidot), t(bcval)
    bc_t = torch.tensor(bc.astype(np.uint8), device="cuda")
    dt = c.advdiff_max_dt(vel_t, kap_t)
    assert dt == pytest.approx(advdiff.max_dt(m, vel, kappa), rel=1e-14)
    po, do = phi.copy(), phidot.copy()
    for _ in range(3):
        c.advdiff_step(dt, vel_t, kap_t, phi_t, pd_t, bc_t, bcv_t, source_q=src_t)
        po, do = advdiff.step(m, dt, vel, kappa, src, bc, bcval, None, po, do)
    np.testing.assert_allclose(phi_t.cpu().numpy(), po, rtol=0, atol=1e-12 * np.abs(po).max())
    np.testing.assert_allclose(pd_t.cpu().numpy(), do, rtol=0, atol=1e-12 * np.abs(do).max())


@pytest.mark.gpu
def test_advection_diffusion_api(gpu):
    import underworld2_gb300 as uw
    res = (12, 10)
    mesh = uw.mesh.FeMesh_Cartesian(elementType="Q1/dQ0", elementRes=res, minCoord=(0.0, 0.0), maxCoord=(1.0, 1.0))
    T = mesh.add_variable(nodeDofCount=1)
    Tdot = mesh.add_variable(nodeDofCount=1)
    v = mesh.add_variable(nodeDofCount=2)
    xy = mesh.data
    T.data[:, 0] = 1.0 - xy[:, 1] + 0.05 * np.cos(np.pi * xy[:, 0]) * np.sin(np.pi * xy[:, 1])
    v.data[:, 0] = np.sin(np.pi * xy[:, 0]) * np.cos(np.pi * xy[:, 1])
    v.data[:, 1] = -np.cos(np.pi * xy[:, 0]) * np.sin(np.pi * xy[:, 1])
    jWalls = mesh.specialSets["MinJ_VertexSet"] + mesh.specialSets["MaxJ_VertexSet"]
    bc = uw.conditions.DirichletCondition(variable=T, indexSetsPerDof=(jWalls,))
    ad = uw.systems.AdvectionDiffusion(phiField=T, phiDotField=Tdot, velocityField=v, fn_diffusivity=1e-2,
                                       conditions=[bc], method="SUPG")
    m = oracle.Mesh(2, 1, res, (0.0, 0.0), (1.0, 1.0))
    kappa = np.full((m.n_el, 9), 1e-2)
    bcmask = bc.mask()[:, 0].astype(bool)
    po, do = T.data[:, 0].copy(), Tdot.data[:, 0].copy()
    bcval = po.copy()
    for _ in range(3):
        dt = ad.get_max_dt()
        assert dt == pytest.approx(advdiff.max_dt(m, v.data, kappa), rel=1e-14)
        ad.integrate(dt)
        po, do = advdiff.step(m, dt, v.data, kappa, None, bcmask, bcval, None, po, do)
    np.testing.assert_allclose(T.data[:, 0], po, rtol=0, atol=1e-12)
    np.testing.assert_allclose(Tdot.data[:, 0], do, rtol=0, atol=1e-10)
