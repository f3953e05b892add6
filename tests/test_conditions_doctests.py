"""Docstring known answers and argument checks of uw.conditions
(P/conditions/_conditions.py:18-170)."""
import numpy as np
import pytest

import underworld2_gb300 as uw


def _setup():
    mesh = uw.mesh.FeMesh_Cartesian(elementType="Q1/dQ0", elementRes=(4, 4), minCoord=(0.0, 0.0), maxCoord=(1.0, 1.0))
    v = uw.mesh.MeshVariable(mesh, 2)
    v.data[:] = [0.0, 0.0]
    return mesh, v


def test_dirichlet_docstring():
    """P/conditions/_conditions.py:93-99: free-slip and no-slip walls."""
    mesh, v = _setup()
    iw = mesh.specialSets["MinI_VertexSet"] + mesh.specialSets["MaxI_VertexSet"]
    jw = mesh.specialSets["MinJ_VertexSet"] + mesh.specialSets["MaxJ_VertexSet"]
    free = uw.conditions.DirichletCondition(v, (iw, jw))
    noslip = uw.conditions.DirichletCondition(v, (iw + jw, iw + jw))
    assert free.mask().sum(0).tolist() == [10, 10]
    assert noslip.mask().sum(0).tolist() == [16, 16]
    assert free.variable is v and free.indexSetsPerDof == (iw, jw)


def test_neumann_docstring():
    """P/conditions/_conditions.py:133-138: a traction on the bottom wall's y dof."""
    mesh, v = _setup()
    bottom = mesh.specialSets["MinJ_VertexSet"]
    c = uw.conditions.NeumannCondition(variable=v, fn_flux=(uw.function.coord()[1], 0.0),
                                       indexSetsPerDof=(None, bottom))
    assert c.mask().sum(0).tolist() == [0, 5]
    c.fn_flux = (1.0, 2.0)
    assert c.fn_flux.evaluate(0.0).tolist() == [[1.0, 2.0]]
    with pytest.raises(ValueError):
        c.fn_flux = "abc"


def test_condition_argument_checks():
    mesh, v = _setup()
    s = mesh.specialSets["MinI_VertexSet"]
    with pytest.raises(TypeError, match="MeshVariable"):
        uw.conditions.DirichletCondition(np.zeros(3), (s, s))
    with pytest.raises(TypeError, match="list or tuple"):
        uw.conditions.DirichletCondition(v, 3)
    with pytest.raises(TypeError, match="'NoneType' or type 'IndexSet'"):
        uw.conditions.DirichletCondition(v, (s, [0, 1]))
    with pytest.raises(ValueError, match="nodeDofCount of 2"):
        uw.conditions.DirichletCondition(v, s)        # one set alone: one dof
    scalar = uw.mesh.MeshVariable(mesh, 1)
    c = uw.conditions.DirichletCondition(scalar, s)
    assert c.indexSetsPerDof == (s,) and c.mask().sum() == 5
    with pytest.raises(TypeError, match="fn_flux"):
        uw.conditions.NeumannCondition(v, (None, s))
    with pytest.raises(AttributeError):
        c.variable = scalar
