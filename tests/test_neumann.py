"""Neumann (flux / traction) conditions: the surface term against the oracle's
loop restatement (CPU), and on the GPU a loaded hydrostatic column and
steady conductive profiles under a boundary flux, whose exact solutions the
elements reproduce (P/conditions/_conditions.py:109-170,
L/Underworld/Utils/src/VectorSurfaceAssemblyTerm_NA__Fn__ni.cpp:163-236)."""
import numpy as np
import pytest
import torch

import underworld2_gb300 as uw
from underworld2_gb300 import systems
from oracle.surface import surface_term


def test_neumann_condition_validation():
    m = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (4, 4), (0.0, 0.0), (1.0, 1.0))
    v = m.add_variable(2)
    with pytest.raises(ValueError):
        uw.conditions.NeumannCondition(v, (m.specialSets["MinJ_VertexSet"],), fn_flux=(1.0, 0.0))
    with pytest.raises(TypeError):
        uw.conditions.NeumannCondition(np.zeros(3), (None, None), fn_flux=(1.0, 0.0))
    c = uw.conditions.NeumannCondition(v, (None, m.specialSets["MinJ_VertexSet"]), fn_flux=(0.0, 1.0))
    assert c.mask().sum(0).tolist() == [0, 5]


@pytest.mark.parametrize("et,res,ng", [("Q1/dQ0", (5, 4), 3), ("Q2/dPc1", (3, 2), 3), ("Q1/dQ0", (3, 2, 2), 2),
                                       ("Q2/dPc1", (2, 2, 1), 3)])
def test_surface_term_matches_oracle(et, res, ng):
    dim = len(res)
    m = uw.mesh.FeMesh_Cartesian(et, res, (0.0,) * dim, (1.0, 2.0, 0.5)[:dim])
    v = m.add_variable(dim)
    ss = m.specialSets
    sets = [ss["MaxJ_VertexSet"] + ss["MinI_VertexSet"], None] + ([ss["MaxK_VertexSet"]] if dim == 3 else [])
    sets[1] = ss["MinJ_VertexSet"]
    x = uw.function.coord()
    fn = tuple(1.0 + 2.0 * x[0] - x[1] * x[d] for d in range(dim))
    c = uw.conditions.NeumannCondition(v, tuple(sets), fn_flux=fn)
    got = systems._surface_flux(c, ng, "cpu").numpy()
    ref = surface_term(m._axes, m._order, c.mask().astype(bool),
                       lambda p: [1.0 + 2.0 * p[0] - p[1] * p[d] for d in range(dim)], ng)
    assert np.abs(got).max() > 0
    np.testing.assert_allclose(got, ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max())
    # a constant flux integrates to flux x wall length / area on each flagged component
    c1 = uw.conditions.NeumannCondition(v, (None, ss["MinJ_VertexSet"]) + ((None,) if dim == 3 else ()),
                                        fn_flux=(0.0, 3.0) + ((0.0,) if dim == 3 else ()))
    tot = systems._surface_flux(c1, ng, "cpu").numpy().reshape(-1, dim).sum(0)
    area = 1.0 * (0.5 if dim == 3 else 1.0)
    np.testing.assert_allclose(tot, [0.0, 3.0 * area] + ([0.0] if dim == 3 else []), atol=1e-13)


@pytest.mark.gpu
@pytest.mark.parametrize("et", ["Q1/dQ0", "Q2/dPc1"])
def test_loaded_hydrostatic_column(et):
    """Free-slip sides, fixed bottom, unit weight downwards and a normal
    traction -P0 on the free top: the discrete solution is exactly u = 0 with
    p = P0 + (1 - y) (cell averages for dQ0, the linear field for dPc1), so the
    pressure level checks the traction's sign and size."""
    P0 = 3.0
    m = uw.mesh.FeMesh_Cartesian(et, (6, 5), (0.0, 0.0), (1.0, 1.0))
    v = m.add_variable(2)
    p = m.subMesh.add_variable(1)
    ss = m.specialSets
    v.data[:] = 0.0
    dbc = uw.conditions.DirichletCondition(v, (ss["MinI_VertexSet"] + ss["MaxI_VertexSet"], ss["MinJ_VertexSet"]))
    nbc = uw.conditions.NeumannCondition(v, (None, ss["MaxJ_VertexSet"]), fn_flux=(0.0, -P0))
    stokes = uw.systems.Stokes(v, p, fn_viscosity=1.0, fn_bodyforce=(0.0, -1.0), conditions=[dbc, nbc])
    solver = uw.systems.Solver(stokes)
    solver.set_inner_rtol(1e-12)
    solver.set_outer_rtol(1e-11)
    solver.solve()
    assert np.abs(v.data).max() < 1e-8
    r = m.elementRes
    xc = (np.arange(r[0]) + 0.5) / r[0]
    yc = (np.arange(r[1]) + 0.5) / r[1]
    cent = np.stack(np.meshgrid(xc, yc, indexing="xy"), -1).reshape(-1, 2)
    pc = p.evaluate(cent)[:, 0]
    np.testing.assert_allclose(pc, P0 + (1.0 - cent[:, 1]), atol=1e-7)


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["SUPG", "SLCN"])
def test_steady_flux_profile(method):
    """T = 0 on top, flux q into the bottom, kappa: steady T = q (1 - y) / kappa."""
    q, kappa = 0.5, 2.0
    m = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (6, 6), (0.0, 0.0), (1.0, 1.0))
    T = m.add_variable(1)
    Tdot = m.add_variable(1)
    vel = m.add_variable(2)
    ss = m.specialSets
    T.data[:] = 0.0
    bc = uw.conditions.DirichletCondition(T, (ss["MaxJ_VertexSet"],))
    nbc = uw.conditions.NeumannCondition(T, (ss["MinJ_VertexSet"],), fn_flux=q)
    ad = uw.systems.AdvectionDiffusion(phiField=T, phiDotField=Tdot if method == "SUPG" else None,
                                       velocityField=vel, fn_diffusivity=kappa, conditions=[bc, nbc],
                                       method=method)
    dt = ad.get_max_dt() if method == "SUPG" else 0.05
    for _ in range(4000 if method == "SUPG" else 400):
        ad.integrate(dt)
    np.testing.assert_allclose(T.data[:, 0], q * (1.0 - m.data[:, 1]) / kappa, atol=1e-6)


@pytest.mark.parametrize("et", ["Q1/dQ0", "Q2/dPc1"])
def test_surface_term_exact_integrals(et):
    """Pins the oracle and the product on a quadratic flux q = 1 + x + x^2 along
    the bottom wall of [0, 2] x [0, 1]: the entries sum to the integral of q
    (partition of unity) and their first moment to the integral of q x
    (isoparametric coordinates), both exact with 3 Gauss points per face."""
    m = uw.mesh.FeMesh_Cartesian(et, (4, 3), (0.0, 0.0), (2.0, 1.0))
    T = m.add_variable(1)
    x = uw.function.coord()
    c = uw.conditions.NeumannCondition(T, (m.specialSets["MinJ_VertexSet"],), fn_flux=1.0 + x[0] + x[0] * x[0])
    ref = surface_term(m._axes, m._order, c.mask().astype(bool), lambda p: [1.0 + p[0] + p[0] ** 2], 3)
    got = systems._surface_flux(c, 3, "cpu").numpy()
    for v in (ref, got):
        assert abs(v.sum() - (2.0 + 2.0 + 8.0 / 3.0)) < 1e-13
        assert abs((v * m.data[:, 0]).sum() - (2.0 + 8.0 / 3.0 + 4.0)) < 1e-13
        assert np.all(v[m.data[:, 1] > 0] == 0.0)
