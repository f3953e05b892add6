"""The uw-compatible API on the GPU, written like the reference's own examples
(docs/examples/04_StokesSinker.ipynb, docs/test/solver_1.py): a sinker on a
free-slip box, solved, then advected; results checked against the oracle."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _sinker(res=(32, 32), ppc=20, inner="mg"):
    import underworld2_gb300 as uw
    mesh = uw.mesh.FeMesh_Cartesian(elementType="Q1/dQ0", elementRes=res, minCoord=(0.0, 0.0), maxCoord=(1.0, 1.0))
    velocityField = mesh.add_variable(nodeDofCount=2)
    pressureField = mesh.subMesh.add_variable(nodeDofCount=1)
    swarm = uw.swarm.Swarm(mesh=mesh)
    material = swarm.add_variable(dataType="int", count=1)
    layout = uw.swarm.layouts.PerCellRandomLayout(swarm=swarm, particlesPerCell=ppc, seed=13)
    swarm.populate_using_layout(layout=layout)
    xy = swarm.particleCoordinates.data
    material.data[:, 0] = (np.sum((xy - [0.5, 0.6]) ** 2, axis=1) < 0.1 ** 2).astype(np.int32)
    fn_visc = uw.function.branching.map(fn_key=material, mapping={0: 1.0, 1: 100.0})
    fn_dens = uw.function.branching.map(fn_key=material, mapping={0: 0.0, 1: 1.0})
    iWalls = mesh.specialSets["MinI_VertexSet"] + mesh.specialSets["MaxI_VertexSet"]
    jWalls = mesh.specialSets["MinJ_VertexSet"] + mesh.specialSets["MaxJ_VertexSet"]
    bc = uw.conditions.DirichletCondition(variable=velocityField, indexSetsPerDof=(iWalls, jWalls))
    stokes = uw.systems.Stokes(velocityField=velocityField, pressureField=pressureField, voronoi_swarm=swarm,
                               conditions=[bc], fn_viscosity=fn_visc, fn_bodyforce=fn_dens * (0.0, -1.0))
    solver = uw.systems.Solver(stokes)
    solver.set_inner_method(inner)
    solver.set_inner_rtol(1e-10)
    solver.set_outer_rtol(1e-9)
    return uw, mesh, velocityField, pressureField, swarm, stokes, solver


@pytest.mark.parametrize("inner", ["mg", "mixed"])
def test_sinker_solve_and_advect(gpu, inner):
    uw, mesh, v, p, swarm, stokes, solver = _sinker(inner=inner)
    solver.solve()
    st = solver.get_stats()
    assert st.residual <= 1e-8
    assert st.pressure_its > 0 and st.velocity_total_its > 0
    # free-slip walls hold
    assert np.all(v.data[mesh.specialSets["MinI_VertexSet"].data, 0] == 0.0)
    assert np.all(v.data[mesh.specialSets["MaxJ_VertexSet"].data, 1] == 0.0)
    # the sinker sinks
    centre = np.argmin(np.sum((mesh.data - [0.5, 0.6]) ** 2, axis=1))
    assert v.data[centre, 1] < 0.0
    r_mom, r_cont = stokes.eqResiduals
    assert r_mom < 1e-7 and r_cont < 1e-7
    vrms = stokes.velocity_rms()
    assert vrms > 0.0
    # advection against the oracle on the same velocity field
    adv = uw.systems.SwarmAdvector(velocityField=v, swarm=swarm, order=2)
    dt = adv.get_max_dt()
    m = oracle.Mesh(2, 1, mesh.elementRes, (0.0, 0.0), (1.0, 1.0))
    x0 = swarm.particleCoordinates.data.copy()
    adv.integrate(dt)
    xo, counts = m.rk2(v.data.ravel(), dt, x0)
    np.testing.assert_array_equal(swarm.particleCoordinates.data, xo)
    np.testing.assert_array_equal(swarm.owningCell.data[:, 0], m.cell_of(xo))


def test_deform_swarm_and_owner(gpu):
    import underworld2_gb300 as uw
    mesh = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (16, 16), (0.0, 0.0), (1.0, 1.0))
    swarm = uw.swarm.Swarm(mesh)
    ret = swarm.add_particles_with_coordinates(np.array([[0.01, 0.01], [0.2, 0.1], [-0.1, -0.1], [0.8, 0.8]]))
    np.testing.assert_array_equal(ret, [0, 1, -1, 2])
    with swarm.deform_swarm():
        swarm.data[0] = [0.1, 0.1]
    assert swarm.owningCell.data[0, 0] == 17          # P/swarm/_swarm.py:629-639
    with pytest.raises(RuntimeError):
        with swarm.deform_swarm():
            swarm.data[1] = [1.5, 0.5]


def test_errors_match_reference(gpu):
    import underworld2_gb300 as uw
    mesh = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (4, 4), (0.0, 0.0), (1.0, 1.0))
    v = mesh.add_variable(2)
    p = mesh.subMesh.add_variable(1)
    with pytest.raises(TypeError):
        uw.systems.Stokes(velocityField=np.zeros(3), pressureField=p, fn_viscosity=1.0)
    with pytest.raises(ValueError):
        uw.systems.Stokes(velocityField=p, pressureField=p, fn_viscosity=1.0)
    with pytest.raises(ValueError):
        uw.systems.Stokes(velocityField=v, pressureField=v, fn_viscosity=1.0)
    st = uw.systems.Stokes(velocityField=v, pressureField=p, fn_viscosity=1.0)
    s = uw.systems.Solver(st)
    with pytest.raises(ValueError):
        s.solve(nonLinearTolerance=-1.0)
    with pytest.raises(ValueError):
        s.set_inner_method("lu")


def test_q2_dpc1_rayleigh_taylor_through_the_api(gpu):
    """The same script shape on a Q2/dPc1 mesh (the reference's Rayleigh-Taylor
    examples use this element pair): solve, residuals, vrms, RK2 against the oracle."""
    import underworld2_gb300 as uw
    res = (16, 16)
    mesh = uw.mesh.FeMesh_Cartesian(elementType="Q2/dPc1", elementRes=res, minCoord=(0.0, 0.0), maxCoord=(1.0, 1.0))
    assert mesh.data.shape == ((2 * res[0] + 1) * (2 * res[1] + 1), 2)
    velocityField = mesh.add_variable(nodeDofCount=2)
    pressureField = mesh.subMesh.add_variable(nodeDofCount=1)
    assert pressureField.data.shape == (3 * res[0] * res[1], 1)
    swarm = uw.swarm.Swarm(mesh=mesh)
    material = swarm.add_variable(dataType="int", count=1)
    swarm.populate_using_layout(layout=uw.swarm.layouts.PerCellRandomLayout(swarm=swarm, particlesPerCell=20, seed=13))
    xy = swarm.particleCoordinates.data
    material.data[:, 0] = (xy[:, 1] > 0.2 + 0.02 * np.cos(np.pi * xy[:, 0])).astype(np.int32)
    fn_visc = uw.function.branching.map(fn_key=material, mapping={0: 0.01, 1: 1.0})
    fn_dens = uw.function.branching.map(fn_key=material, mapping={0: 0.0, 1: 1.0})
    iWalls = mesh.specialSets["MinI_VertexSet"] + mesh.specialSets["MaxI_VertexSet"]
    jWalls = mesh.specialSets["MinJ_VertexSet"] + mesh.specialSets["MaxJ_VertexSet"]
    bc = uw.conditions.DirichletCondition(variable=velocityField, indexSetsPerDof=(iWalls, jWalls))
    stokes = uw.systems.Stokes(velocityField=velocityField, pressureField=pressureField, voronoi_swarm=swarm,
                               conditions=[bc], fn_viscosity=fn_visc, fn_bodyforce=fn_dens * (0.0, -1.0))
    solver = uw.systems.Solver(stokes)
    solver.set_inner_method("mixed")
    solver.set_inner_rtol(1e-10)
    solver.set_outer_rtol(1e-9)
    solver.solve()
    st = solver.get_stats()
    assert st.residual <= 1e-8
    r_mom, r_cont = stokes.eqResiduals
    assert r_mom < 1e-7 and r_cont < 1e-7
    assert stokes.velocity_rms() > 0.0
    adv = uw.systems.SwarmAdvector(velocityField=velocityField, swarm=swarm, order=2)
    dt = adv.get_max_dt()
    m = oracle.Mesh(2, 2, res, (0.0, 0.0), (1.0, 1.0), porder=1)
    x0 = swarm.particleCoordinates.data.copy()
    adv.integrate(dt)
    xo, counts = m.rk2(velocityField.data.ravel(), dt, x0)
    np.testing.assert_array_equal(swarm.particleCoordinates.data, xo)
