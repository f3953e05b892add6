"""uw.function.analytic: the Dohrmann & Bochev fixed-wall Stokes solutions
(P/function/analytic.py:568-656), CPU.

The fields are checked against their definitions by central differences:
divergence-free velocity, strain rate = symmetric velocity gradient, stress =
2 eta strain rate, body force = -div(2 eta strain rate) + grad p.  The 2D body
force is also compared with the reference's closed form at a point, and
get_bcs with the reference's wall-flux normalisation on a small mesh."""
import numpy as np
import pytest

import underworld2_gb300 as uw
from underworld2_gb300 import function as fn

H = 1e-5


def _fd(f, x, d):
    e = np.zeros_like(x)
    e[:, d] = H
    return (f.evaluate(x + e) - f.evaluate(x - e)) / (2 * H)


def _sym_index(dim):
    # symmetric-tensor component order: xx, yy[, zz], xy[, xz, yz]
    if dim == 2:
        return {(0, 0): 0, (1, 1): 1, (0, 1): 2, (1, 0): 2}
    return {(0, 0): 0, (1, 1): 1, (2, 2): 2, (0, 1): 3, (1, 0): 3, (0, 2): 4, (2, 0): 4, (1, 2): 5, (2, 1): 5}


@pytest.mark.parametrize("sol,dim", [(lambda: fn.analytic.SolDB2d(), 2), (lambda: fn.analytic.SolDB3d(), 3),
                                     (lambda: fn.analytic.SolDB3d(Beta=1.5), 3)])
def test_fields_satisfy_stokes(sol, dim):
    s = sol()
    x = np.random.default_rng(3).uniform(0.05, 0.95, (40, dim))
    grad_u = np.stack([_fd(s.fn_velocity, x, d) for d in range(dim)], 2)    # [n, i, d] = du_i/dx_d
    assert np.abs(np.trace(grad_u, axis1=1, axis2=2)).max() < 1e-7
    sr = s.fn_strainRate.evaluate(x)
    idx = _sym_index(dim)
    for (i, j), k in idx.items():
        np.testing.assert_allclose(sr[:, k], 0.5 * (grad_u[:, i, j] + grad_u[:, j, i]), atol=1e-7)
    eta = s.fn_viscosity.evaluate(x)
    np.testing.assert_allclose(s.fn_stress.evaluate(x), 2.0 * eta * sr, rtol=1e-13)
    div_tau = np.zeros((len(x), dim))
    for d in range(dim):
        dtau = _fd(s.fn_stress, x, d)
        for i in range(dim):
            div_tau[:, i] += dtau[:, idx[(i, d)]]
    grad_p = np.concatenate([_fd(s.fn_pressure, x, d) for d in range(dim)], 1)
    np.testing.assert_allclose(s.fn_bodyforce.evaluate(x), -div_tau + grad_p, atol=1e-5)


def test_db2d_closed_form_body_force():
    # the reference's printed body force at (0.3, 0.7): (-z - 1 + 3x^2 z^2, -1 + 3x + 2x^3 z)
    f = fn.analytic.SolDB2d().fn_bodyforce.evaluate((0.3, 0.7))
    np.testing.assert_allclose(f, [[-1.5677, -0.0622]], rtol=0, atol=1e-12)


def test_get_bcs_matches_wall_fluxes():
    s = fn.analytic.SolDB2d()
    mesh = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (6, 5), (0.0, 0.0), (1.0, 1.0))
    v = mesh.add_variable(2)
    bc = s.get_bcs(v)
    ss = mesh.specialSets
    for ax, name in ((0, "I"), (1, "J")):
        for side in ("Min", "Max"):
            verts = ss["%s%s_VertexSet" % (side, name)]
            idx = verts.data
            # flux of the interpolant of the nodal values: trapezoid weights along the wall
            other = mesh.data[idx, 1 - ax]
            order = np.argsort(other)
            c, vv = other[order], v.data[idx, ax][order]
            num = float(np.sum(0.5 * (vv[1:] + vv[:-1]) * np.diff(c)))
            ana = uw.utils.Integral(s.fn_velocity[ax], mesh, integrationType="surface",
                                    surfaceIndexSet=verts).evaluate()
            assert abs(num - float(np.ravel(ana)[0])) < 1e-12
    walls = ss["AllWalls_VertexSet"].data
    # tangential components keep the analytic values exactly
    ana = s.fn_velocity.evaluate(mesh.data[walls])
    on_x_walls = np.isin(walls, np.concatenate([ss["MinI_VertexSet"].data, ss["MaxI_VertexSet"].data]))
    np.testing.assert_array_equal(v.data[walls][~on_x_walls, 0], ana[~on_x_walls, 0])
    assert bc is not None
