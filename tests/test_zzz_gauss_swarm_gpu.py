"""Swarm variables on a Gauss integration swarm (GPU, through the C ABI and the
uw-style API): each Gauss point takes the value of the nearest particle of its
element, as GeneralSwarm_IntegrationPointMap finds it
(L/PICellerator/MaterialPoints/src/GeneralSwarm.cpp:319-431), checked against
the oracle's restatement (oracle.Mesh.gauss_nearest); then a Stokes system
without a voronoi swarm whose functions read a swarm variable, the case of the
reference's Rayleigh-Taylor example, against the oracle's direct solve.  The
same map drives tests/test_rayleigh_taylor_known_answer.py on the CPU."""
import numpy as np
import pytest
import torch

import oracle
from tests import analytic_convergence as ac
from tests import oracle_system as osys

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,order,res", [(2, 1, (6, 5)), (3, 1, (3, 3, 2)), (2, 2, (4, 3))])
def test_gauss_nearest_matches_oracle(gpu, dim, order, res):
    from underworld2_gb300._core import Context, rng_seed
    c = Context(dim, res, (0.0,) * dim, (1.0,) * dim, order=order, porder=order - 1)
    ppc = 7
    x, owner, off, lst, _ = c.layout_random(ppc, rng_seed(13))
    m = oracle.Mesh(dim, order, res, (0.0,) * dim, (1.0,) * dim, porder=order - 1)
    xo, _ = m.layout_random(ppc, 13)
    np.testing.assert_array_equal(x.cpu().numpy(), xo)
    tbl, cnt, _ = m.initial_tables(ppc, ppc)
    ng = 3 if order == 1 else 5
    xi, _ = m.gauss_points(ng)
    pid = c.gauss_nearest(torch.from_numpy(xi), off, lst, x).cpu().numpy().reshape(m.n_el, len(xi))
    np.testing.assert_array_equal(pid, m.gauss_nearest(xo, tbl, cnt, xi))


def test_stokes_on_gauss_swarm_with_swarm_variables(gpu):
    import underworld2_gb300 as uw
    res = (16, 16)
    mesh = uw.mesh.FeMesh_Cartesian(elementType="Q1/dQ0", elementRes=res, minCoord=(0.0, 0.0), maxCoord=(1.0, 1.0))
    velocityField = mesh.add_variable(nodeDofCount=2)
    pressureField = mesh.subMesh.add_variable(nodeDofCount=1)
    swarm = uw.swarm.Swarm(mesh=mesh)
    material = swarm.add_variable(dataType="int", count=1)
    swarm.populate_using_layout(layout=uw.swarm.layouts.PerCellRandomLayout(swarm=swarm, particlesPerCell=12, seed=13))
    xy = swarm.particleCoordinates.data.copy()
    material.data[:, 0] = (xy[:, 1] > 0.2 + 0.02 * np.cos(np.pi * xy[:, 0])).astype(np.int32)
    fn_visc = uw.function.branching.map(fn_key=material, mapping={0: 0.1, 1: 1.0})
    fn_dens = uw.function.branching.map(fn_key=material, mapping={0: 0.0, 1: 1.0})
    iWalls = mesh.specialSets["MinI_VertexSet"] + mesh.specialSets["MaxI_VertexSet"]
    jWalls = mesh.specialSets["MinJ_VertexSet"] + mesh.specialSets["MaxJ_VertexSet"]
    bc = uw.conditions.DirichletCondition(variable=velocityField, indexSetsPerDof=(iWalls, jWalls))
    stokes = uw.systems.Stokes(velocityField=velocityField, pressureField=pressureField, conditions=[bc],
                               fn_viscosity=fn_visc, fn_bodyforce=fn_dens * (0.0, -1.0))
    solver = uw.systems.Solver(stokes)
    solver.set_inner_rtol(1e-11)
    solver.set_outer_rtol(1e-10)
    solver.solve()
    # oracle: the same Gauss points, materials of the nearest particles, direct solve
    m = oracle.Mesh(2, 1, res, (0.0, 0.0), (1.0, 1.0))
    tbl, cnt, _ = m.initial_tables(12, 12)
    g = ac._Rule(m, 3)
    nq = len(g.w)
    pid = m.gauss_nearest(xy, tbl, cnt, g.xi).ravel()
    mat = material.data[:, 0][pid]
    eta = np.where(mat == 1, 1.0, 0.1)
    body = np.zeros((m.n_el * nq, 2))
    body[:, 1] = -np.where(mat == 1, 1.0, 0.0)
    X = m.node_coords()[:, :2]
    mask = np.zeros(m.n_nodes * 2, np.uint8)
    for d in range(2):
        mask[np.flatnonzero(np.isclose(X[:, d], 0.0) | np.isclose(X[:, d], 1.0)) * 2 + d] = 1
    pts = [(e * nq + np.arange(nq), g.xi, g.w) for e in range(m.n_el)]
    uo, po = osys.solve(osys.assemble(m, pts, eta, body, mask, np.zeros(m.n_nodes * 2)), m.n_nodes * 2)
    u = velocityField.data.ravel()
    assert np.linalg.norm(u - uo) / np.linalg.norm(uo) < 1e-8
    p = pressureField.data[:, 0]
    p, po = p - p.mean(), po - po.mean()
    assert np.linalg.norm(p - po) / np.linalg.norm(po) < 1e-8


def test_swarm_variable_at_coordinates_takes_nearest_particle(gpu):
    """docs/user_guide/04_Functions.ipynb: a swarm variable evaluated at plain
    coordinates returns its nearest particle's value (the guide expects particle 1
    at (0.4, 0.4) for the point (0.5, 0.5)); integer variables stay integers."""
    import underworld2_gb300 as uw
    mesh = uw.mesh.FeMesh_Cartesian(maxCoord=(2.0, 1.0))
    swarm = uw.swarm.Swarm(mesh)
    swarm.add_particles_with_coordinates(np.array([(0.1, 0.1), (0.4, 0.4), (0.9, 0.9), (1.0, 0.1), (1.9, 0.1)]))
    index_var = swarm.add_variable("int", 1)
    index_var.data[:, 0] = np.arange(swarm.particleLocalCount)
    result = index_var.evaluate((0.5, 0.5))
    assert result.dtype == np.int32 and result.tolist() == [[1]]
    pts = np.array([[1.8, 0.0], [0.1, 0.11], [0.95, 0.8]])
    d2 = ((pts[:, None, :] - swarm.data[None, :, :]) ** 2).sum(-1)
    np.testing.assert_array_equal(index_var.evaluate(pts)[:, 0], np.argmin(d2, axis=1))
    np.testing.assert_array_equal(index_var.evaluate(swarm)[:, 0], np.arange(5))


def test_swarm_variable_types_evaluate_and_checkpoint(gpu, tmp_path):
    """docs/test/swarmvariable_types.ipynb: variables of every type hold their
    type's largest value, evaluate to it at (0.5, 0.5) (nearest particle), and
    survive a save / load onto a new swarm."""
    import underworld2_gb300 as uw
    mesh = uw.mesh.FeMesh_Cartesian()

    def addvars(sw):
        return ((sw.add_variable("char", 1), np.iinfo(np.int8).max), (sw.add_variable("short", 1), np.iinfo(np.int16).max),
                (sw.add_variable("int", 1), np.iinfo(np.int32).max), (sw.add_variable("long", 1), np.iinfo(np.int64).max),
                (sw.add_variable("float", 1), np.finfo(np.float32).max),
                (sw.add_variable("double", 1), np.finfo(np.float64).max))

    swarm = uw.swarm.Swarm(mesh)
    vars1 = addvars(swarm)
    swarm.populate_using_layout(uw.swarm.layouts.PerCellSpaceFillerLayout(swarm, 20))
    for v, mx in vars1:
        v.data[:] = mx
    for v, mx in vars1:
        res = v.evaluate((0.5, 0.5))
        assert res.dtype == v.data.dtype and res.tolist() == [[mx]]
    swarm.save(str(tmp_path / "swarm.h5"))
    for i, (v, _) in enumerate(vars1):
        v.save(str(tmp_path / ("var%d.h5" % i)))
    swarm2 = uw.swarm.Swarm(mesh)
    vars2 = addvars(swarm2)
    swarm2.load(str(tmp_path / "swarm.h5"))
    for i, (v, mx) in enumerate(vars2):
        v.load(str(tmp_path / ("var%d.h5" % i)))
        assert np.all(v.data == mx)


def test_integral_of_swarm_variable_map():
    """P/function/branching.py:72-100: a swarm variable marking the particles in
    the unit circle, mapped to 1 (and with a default), integrates to pi within 2 %
    over [-1, 1]^2 (8 x 8 Q1, 20 space-filler particles per cell): the Gauss
    points read their elements' nearest particles."""
    import underworld2_gb300 as uw
    fn = uw.function
    mesh = uw.mesh.FeMesh_Cartesian(elementRes=(8, 8), minCoord=(-1.0, -1.0), maxCoord=(1.0, 1.0))
    swarm = uw.swarm.Swarm(mesh)
    svar = swarm.add_variable("int", 1)
    swarm.populate_using_layout(uw.swarm.layouts.PerCellSpaceFillerLayout(swarm, 20))
    svar.data[:] = 0
    xy = swarm.particleCoordinates.data
    svar.data[(xy ** 2).sum(1) < 1.0, 0] = 1
    fn_map = fn.branching.map(fn_key=svar, mapping={0: 0.0, 1: 1.0})
    assert np.allclose(np.pi, uw.utils.Integral(fn_map, mesh).evaluate(), rtol=2e-2)
    fn_map = fn.branching.map(fn_key=svar, mapping={1: 1.0}, fn_default=0.0)
    assert np.allclose(np.pi, uw.utils.Integral(fn_map, mesh).evaluate(), rtol=2e-2)


def test_fn_particle_found():
    """P/swarm/_swarm.py:430-466: fn_particle_found is True at the swarm's own
    particles, False at a plain coordinate, and at Gauss points True exactly in
    the elements that still hold a particle after those outside the unit circle
    escaped; the area of those elements (counted here from the 2 x 2 Gauss
    layout's positions) is the integral, and it is pi/4 within 2 %."""
    import underworld2_gb300 as uw
    mesh = uw.mesh.FeMesh_Cartesian(elementRes=(32, 32))
    swarm = uw.swarm.Swarm(mesh, particleEscape=True)
    swarm.populate_using_layout(uw.swarm.layouts.PerCellGaussLayout(swarm, 2))
    fn_pf = swarm.fn_particle_found()
    assert fn_pf.evaluate(swarm).all()
    r = fn_pf.evaluate((0.3, 0.9))
    assert r.dtype == bool and r.tolist() == [[False]]
    with swarm.deform_swarm():
        for ind, coord in enumerate(swarm.data):
            if np.dot(coord, coord) > 1.0:
                swarm.data[ind] = (99999.0, 99999.0)
    xy = swarm.particleCoordinates.data
    assert (xy ** 2).sum(1).max() <= 1.0
    cells = np.unique(np.minimum((xy * 32).astype(np.int64), 31) @ np.array([1, 32]))
    incirc = uw.function.branching.conditional(((fn_pf, 1.0), (True, 0.0)))
    val = uw.utils.Integral(incirc, mesh).evaluate()
    np.testing.assert_allclose(val, [len(cells) / 32.0 ** 2], rtol=1e-12)
    assert np.isclose(val, np.pi / 4.0, rtol=2e-2).all()
