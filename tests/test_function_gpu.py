"""Mesh-variable inputs of the function graph on the GPU (uwg_interpolate_field):
the reference docstring's known answers for MeshVariable.evaluate
(P/function/_function.py:864-905), values bit-exact with the velocity
interpolation of the particle path, exact gradients of fields the element
reproduces, and strain-rate invariants built from fn_gradient."""
import numpy as np
import pytest
import torch

import oracle
import underworld2_gb300 as uw

pytestmark = pytest.mark.gpu


def test_meshvariable_evaluate_docstring(gpu):
    mesh = uw.mesh.FeMesh_Cartesian()
    var = uw.mesh.MeshVariable(mesh, 1)
    var.data[:, 0] = np.linspace(0, 1, len(var.data))
    assert np.allclose(var.evaluate((0.2, 0.5)), np.array([[0.45]]))
    locations = np.zeros((10, 2))
    locations[:, 0] = 0.5
    locations[:, 1] = np.linspace(0.0, 1.0, 10)
    expect = np.array([[0.08333333], [0.17592593], [0.26851852], [0.36111111], [0.4537037], [0.5462963],
                       [0.63888889], [0.73148148], [0.82407407], [0.91666667]])
    assert np.allclose(var.evaluate(locations), expect)
    assert np.allclose(var.evaluate(mesh), var.evaluate(mesh.data))
    assert var.evaluate(np.zeros((0, 2))).shape == (0, 1)


@pytest.mark.parametrize("dim,order,res", [(2, 1, (7, 5)), (3, 1, (4, 3, 5)), (2, 2, (5, 4))])
def test_interpolate_field_values_and_gradients(gpu, dim, order, res):
    from underworld2_gb300._core import Context
    c = Context(dim, res, (0.0,) * dim, (1.0,) * dim, order=order, porder=1 if order == 2 else 0)
    m = oracle.Mesh(dim, order, res, (0.0,) * dim, (1.0,) * dim, porder=1 if order == 2 else 0)
    rng = np.random.default_rng(2)
    nodes = m.node_coords()
    vel = rng.standard_normal((m.n_nodes, dim))
    pts = rng.uniform(0.0, 1.0, (200, dim))
    pts[:5] = nodes[rng.integers(0, m.n_nodes, 5)]
    t = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    val, _ = c.interpolate_field(t(pts), t(vel.ravel()), dim)
    ref = np.array([m.interpolate(vel, p) for p in pts])
    np.testing.assert_array_equal(val.cpu().numpy(), ref)
    # a field the element reproduces exactly (linear; quadratic in x for Q2) has exact gradients
    A = rng.standard_normal((3, dim))
    f = nodes @ A.T + (0.7 * nodes[:, :1] ** 2 if order == 2 else 0.0)
    v, g = c.interpolate_field(t(pts), t(f.ravel()), 3, grad=True)
    gexp = np.broadcast_to(A, (len(pts), 3, dim)).copy()
    if order == 2:
        gexp[:, :, 0] += 1.4 * pts[:, :1]
    np.testing.assert_allclose(g.cpu().numpy(), gexp, rtol=0, atol=1e-12)
    np.testing.assert_allclose(v.cpu().numpy(), pts @ A.T + (0.7 * pts[:, :1] ** 2 if order == 2 else 0.0),
                               rtol=0, atol=1e-12)
    out, _ = c.interpolate_field(t(np.array([[1.5] * dim])), t(f.ravel()), 3)
    assert torch.isnan(out).all()


def test_strain_rate_invariant_from_fn_gradient(gpu):
    mesh = uw.mesh.FeMesh_Cartesian(elementRes=(8, 6), minCoord=(0.0, 0.0), maxCoord=(2.0, 1.0))
    v = mesh.add_variable(nodeDofCount=2)
    xy = mesh.data
    L = np.array([[0.3, 1.2], [-0.5, -0.3]])
    v.data[...] = xy @ L.T
    sr = uw.function.tensor.symmetric(v.fn_gradient)
    pts = np.random.default_rng(0).uniform((0.0, 0.0), (2.0, 1.0), (50, 2))
    S = 0.5 * (L + L.T)
    np.testing.assert_allclose(v.fn_gradient.evaluate(pts), np.broadcast_to(L.ravel(), (50, 4)), atol=1e-12)
    np.testing.assert_allclose(sr.evaluate(pts), np.broadcast_to([S[0, 0], S[1, 1], S[0, 1]], (50, 3)), atol=1e-12)
    inv = uw.function.tensor.second_invariant(sr).evaluate(pts)
    np.testing.assert_allclose(inv, np.sqrt(0.5 * (S * S).sum()), rtol=1e-12)
    T = mesh.add_variable(nodeDofCount=1)
    T.data[:, 0] = 1.0 - xy[:, 1]
    eta = uw.function.math.exp(-2.0 * T)
    np.testing.assert_allclose(eta.evaluate(pts), np.exp(-2.0 * (1.0 - pts[:, 1:2])), rtol=1e-12)
    np.testing.assert_allclose(T.fn_gradient.evaluate(pts), np.broadcast_to([0.0, -1.0], (50, 2)), atol=1e-12)
