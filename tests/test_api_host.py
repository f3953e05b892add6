"""Host-side parts of the uw-style API that need no GPU: solver options and
statistics objects before a solve (P/systems/_bsscr.py:509-512,704-738)."""
import underworld2_gb300 as uw


def test_solver_option_setters_and_stats(capsys):
    m = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (4, 4), (0.0, 0.0), (1.0, 1.0))
    v = m.add_variable(2)
    p = m.subMesh.add_variable(1)
    solver = uw.systems.Solver(uw.systems.Stokes(v, p, fn_viscosity=1.0))
    a = solver.get_nonLinearStats()
    assert a.picard_iterations == 0 and a.picard_residual == 0.0
    solver.set_inner_method("mixed")
    solver.set_inner_rtol(1e-9)
    solver.set_outer_rtol(1e-8)
    solver.print_petsc_options()
    out = capsys.readouterr().out
    assert "inner_method=mixed" in out and "inner_rtol=1e-09" in out and "outer_rtol=1e-08" in out


def test_property_members():
    import numpy as np
    m = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (4, 4), (0.0, 0.0), (1.0, 1.0))
    v = m.add_variable(2)
    v.data[:, 0] = np.arange(v.data.shape[0])
    c = v.copy()
    assert c.nodeDofCount == 2 and c.mesh is m and np.all(c.data == 0.0)
    d = v.copy(deepcopy=True)
    np.testing.assert_array_equal(d.data, v.data)
    assert v.dataType == "double" and v.syncronise() is None
    p = m.subMesh.add_variable(1)
    st = uw.systems.Stokes(v, p, fn_viscosity=1.0)
    assert st.fn_one_on_lambda is None and st.fn_source is None
    st.fn_one_on_lambda = 1e-3
    assert isinstance(st.fn_one_on_lambda, uw.function.Function)
    sw = uw.swarm.Swarm(m)
    a = sw.add_variable("int", 1)
    b = a.copy()
    assert sw.variables == [a, b] and b.dataType == "int" and b.count == 1
    adv = uw.systems.SwarmAdvector(v, sw)
    assert adv.dt == 0.0 and adv.time == 0.0
    adv.time = 2.5
    assert adv.time == 2.5


def test_penalty_option_and_compressibility_warning(capsys):
    """docs/test/solver_penalty_test.py: a penalty on a compressible system draws
    the reference's warning at solve() (P/systems/_bsscr.py:320-321,359-365);
    set_penalty switches the Schur preconditioner name as the reference does
    (:766-780).  The warning comes before any device work, so the solve's own
    failure on a machine without a GPU follows it."""
    import pytest
    import torch
    m = uw.mesh.FeMesh_Cartesian("Q1/DQ0", (2, 2), (0.0, 0.0), (1.0, 1.0))
    v = uw.mesh.MeshVariable(m, 2)
    p = uw.mesh.MeshVariable(m.subMesh, 1)
    solver = uw.systems.Solver(uw.systems.Stokes(v, p, 1.0, (0.0, 0.0), fn_one_on_lambda=1.0))
    solver.set_penalty(1.0)
    assert solver.options.main.penalty == 1.0 and solver.options.main.Q22_pc_type == "gkgdiag"
    if not torch.cuda.is_available():
        with pytest.warns(UserWarning) as w:
            with pytest.raises(RuntimeError):
                solver.solve()
        assert str(w[0].message) == uw.systems.StokesSolver._warning_penalty_compressibility
    solver.set_penalty(-1.0)
    assert solver.options.main.penalty == 0.0 and "Invalid penalty" in capsys.readouterr().out
