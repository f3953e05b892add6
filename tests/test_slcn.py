"""SLCN advection-diffusion (the reference's AdvectionDiffusion, method "SLCN").

CPU: the oracle's departure values reproduce a linear field moved by a uniform
velocity (cubic stencils are exact for it), and its Crank-Nicolson solve keeps
a steady linear profile.  GPU: departure values bit-exact with the oracle
(uwo_slcn_phistar), the diffusion solve within 1e-10 of the oracle's direct
solve, and the uw-style ``AdvectionDiffusion(method="SLCN")`` over several
steps against the oracle's step.
"""
import numpy as np
import pytest
import torch

import oracle
from oracle import slcn


def _cellular(nodes, dim, amp=1.0):
    v = np.zeros((len(nodes), dim))
    s, c = np.sin(np.pi * nodes), np.cos(np.pi * nodes)
    v[:, 0] = amp * s[:, 0] * c[:, dim - 1]
    v[:, dim - 1] = -amp * c[:, 0] * s[:, dim - 1]
    if dim == 3:
        v[:, 1] = 0.3 * amp * s[:, 1] * c[:, 0]
    return v


def test_oracle_departure_linear_field_uniform_velocity():
    m = oracle.Mesh(2, 1, (8, 6), (0.0, 0.0), (2.0, 1.0))
    nodes = m.node_coords()
    vel = np.tile([0.3, -0.2], (m.n_nodes, 1))
    phi = 0.5 + 1.5 * nodes[:, 0] - 0.7 * nodes[:, 1]
    dt = 0.9
    ps = m.slcn_phistar(vel, phi, dt)
    # RK4 with a uniform field: x - INV6 dt 6 v, INV6 = 0.166666666667, clamped to the box
    back = nodes - 0.166666666667 * dt * 6.0 * vel[0]
    back[:, 0] = np.clip(back[:, 0], 0.0, 2.0)
    back[:, 1] = np.clip(back[:, 1], 0.0, 1.0)
    np.testing.assert_allclose(ps, 0.5 + 1.5 * back[:, 0] - 0.7 * back[:, 1], rtol=0, atol=1e-12)


def test_oracle_crank_nicolson_keeps_linear_profile():
    m = oracle.Mesh(2, 1, (6, 5), (0.0, 0.0), (1.0, 1.0))
    nodes = m.node_coords()
    bc = np.isclose(nodes[:, 1], 0.0) | np.isclose(nodes[:, 1], 1.0)
    phi = 1.0 - nodes[:, 1]
    kappa = np.full((m.n_el, 25), 0.3)
    out = slcn.solve(m, 0.05, kappa, None, bc, phi, phi)
    np.testing.assert_allclose(out, phi, rtol=0, atol=1e-13)


def _case(dim, res, seed):
    rng = np.random.default_rng(seed)
    m = oracle.Mesh(dim, 1, res, (0.0,) * dim, (1.0,) * dim)
    nodes = m.node_coords()
    vel = _cellular(nodes, dim) + 0.05 * rng.standard_normal((m.n_nodes, dim))
    phi = 1.0 - nodes[:, dim - 1] + 0.2 * np.sin(3.0 * nodes[:, 0] + 1.0) * np.cos(2.0 * nodes[:, dim - 1])
    nq = 5 ** dim
    kappa = rng.uniform(1e-3, 5e-2, (m.n_el, nq))
    src = rng.uniform(-0.5, 0.5, (m.n_el, nq))
    bc = np.isclose(nodes[:, dim - 1], 0.0) | np.isclose(nodes[:, dim - 1], 1.0)
    return m, vel, phi, kappa, src, bc


@pytest.mark.gpu
@pytest.mark.parametrize("dim,res", [(2, (12, 10)), (3, (6, 5, 5))])
def test_slcn_departure_bit_exact(gpu, dim, res):
    from underworld2_gb300._core import Context
    m, vel, phi, *_ = _case(dim, res, 3)
    c = Context(dim, res, (0.0,) * dim, (1.0,) * dim)
    assert c.min_sep == m.min_sep()
    vt, pt = torch.tensor(vel.ravel(), device="cuda"), torch.tensor(phi, device="cuda")
    for dt in (0.0, 1e-9, 0.05, 0.4):
        ps = c.slcn_phistar(dt, vt, pt).cpu().numpy()
        np.testing.assert_array_equal(ps, m.slcn_phistar(vel, phi, dt))


@pytest.mark.gpu
@pytest.mark.parametrize("dim,res", [(2, (12, 10)), (3, (6, 5, 5))])
@pytest.mark.parametrize("with_source", [False, True])
def test_slcn_solve_matches_direct(gpu, dim, res, with_source):
    from underworld2_gb300._core import Context
    m, vel, phi, kappa, src, bc = _case(dim, res, 4)
    src = src if with_source else None
    c = Context(dim, res, (0.0,) * dim, (1.0,) * dim)
    dt = 0.05
    ps = m.slcn_phistar(vel, phi, dt)
    t = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    phi_t = t(phi)
    its, res_ = c.slcn_solve(dt, t(kappa.ravel()), torch.tensor(bc.astype(np.uint8)), t(ps), phi_t,
                             source_q=None if src is None else t(src.ravel()), rtol=1e-13)
    assert res_ <= 1e-13 and its > 0
    ref = slcn.solve(m, dt, kappa, src, bc, ps, phi)
    np.testing.assert_allclose(phi_t.cpu().numpy(), ref, rtol=0, atol=1e-10 * np.abs(ref).max())


@pytest.mark.gpu
def test_slcn_rejects_small_meshes(gpu):
    from underworld2_gb300 import _native
    from underworld2_gb300._core import Context
    c = Context(2, (2, 6), (0.0, 0.0), (1.0, 1.0))
    z = torch.zeros(c.n_nodes * 2, dtype=torch.float64, device="cuda")
    with pytest.raises(_native.UwgError):
        c.slcn_phistar(0.1, z, z[: c.n_nodes].contiguous())


@pytest.mark.gpu
def test_advection_diffusion_slcn_api(gpu):
    import underworld2_gb300 as uw
    res = (16, 12)
    mesh = uw.mesh.FeMesh_Cartesian(elementType="Q1/dQ0", elementRes=res, minCoord=(0.0, 0.0), maxCoord=(1.0, 1.0))
    T = mesh.add_variable(nodeDofCount=1)
    v = mesh.add_variable(nodeDofCount=2)
    xy = mesh.data
    T.data[:, 0] = 1.0 - xy[:, 1] + 0.05 * np.cos(np.pi * xy[:, 0]) * np.sin(np.pi * xy[:, 1])
    v.data[...] = _cellular(xy, 2, amp=20.0)
    walls = mesh.specialSets["MinJ_VertexSet"] + mesh.specialSets["MaxJ_VertexSet"]
    bc = uw.conditions.DirichletCondition(variable=T, indexSetsPerDof=(walls,))
    kappa = 1e-2 * (1.0 + uw.function.input()[0])
    ad = uw.systems.AdvectionDiffusion(phiField=T, velocityField=v, fn_diffusivity=kappa, conditions=[bc],
                                       method="SLCN")
    m = oracle.Mesh(2, 1, res, (0.0, 0.0), (1.0, 1.0))
    gx = slcn.gauss_coords(m)
    kq = 1e-2 * (1.0 + gx[:, :, 0])
    bcmask = bc.mask()[:, 0].astype(bool)
    po = T.data[:, 0].copy()
    for _ in range(3):
        dt = ad.get_max_dt()
        assert dt == pytest.approx(slcn.max_dt(m, v.data, 1e-2 * (1.0 + xy[:, 0])), rel=1e-14)
        ad.integrate(dt)
        po, _ = slcn.step(m, dt, v.data, kq, None, bcmask, po)
        np.testing.assert_allclose(T.data[:, 0], po, rtol=0, atol=1e-9)
