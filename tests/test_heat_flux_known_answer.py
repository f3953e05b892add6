"""Known answer of the reference's advection-diffusion test with a boundary flux
(docs/test/HeatEq_fluxBC.ipynb).

A 2D 10 x 15 Q1 mesh on [0, 1] x [-0.6, 1.3], diffusivity k = 6.70, source
h = 8.0, velocity (0, 2.47), temperature TD = 8 on one horizontal wall and a
flux of magnitude 4 (NeumannCondition with fn_flux = n_y * 4, n_y the outward
normal) through the other, integrated from T = TD until the relative change
per step falls below 1e-5 (at most 2000 steps) with dt = get_max_dt() for SUPG
and 5 get_max_dt() for SLCN.  The reference requires the steady state to lie
within 1 % (relative L2 norm) of the analytic solution
T(y) = c0 exp(v y / k) + h y / v + c1 for both wall arrangements and both
methods.  Run here through the oracle restatements; the GPU kernels are checked
against the same restatements in tests/test_advdiff.py and tests/test_slcn.py.
"""
import numpy as np
import pytest

import oracle
from oracle import advdiff, slcn
from oracle.surface import surface_term

TD, K, H, PHI, V = 8.0, 6.70, 8.0, 4.0, 2.47
Y0, Y1 = -0.6, 1.3


def _analytic(wall):
    if wall == "a":   # flux through the top (outward normal +y), Dirichlet at the bottom
        c0 = (PHI / K - H / V) * K / V * np.exp(-V / K * Y1)
        c1 = TD - c0 * np.exp(V / K * Y0) - H / V * Y0
        return 1.0, c0, c1
    c0 = (PHI / K - H / V) * K / V * np.exp(-V / K * Y0)
    c1 = TD - c0 * np.exp(V / K * Y1) - H / V * Y1
    return -1.0, c0, c1


def _percent_error(m, T, c0, c1):
    """100 ||T_a - T|| / ||T_a|| over the mesh, 5-point Gauss rule per axis."""
    N, _, w = slcn._shapes(m)
    yq = slcn.gauss_coords(m)[:, :, 1]
    num = den = 0.0
    for e in range(m.n_el):
        nodes = m.element_nodes(e)
        idx = slcn._elem_index(m, e)
        det = np.prod([0.5 * (m.axes[d][idx[d] + 1] - m.axes[d][idx[d]]) for d in range(2)])
        ta = c0 * np.exp(V / K * yq[e]) + H / V * yq[e] + c1
        tq = N @ T[nodes]
        num += float(np.sum(w * det * (ta - tq) ** 2))
        den += float(np.sum(w * det * ta ** 2))
    return 100.0 * np.sqrt(num / den)


@pytest.mark.parametrize("method", ["supg", "slcn"])
@pytest.mark.parametrize("wall", ["a", "b"])
def test_steady_state_within_one_percent(wall, method):
    m = oracle.Mesh(2, 1, (10, 15), (0.0, Y0), (1.0, Y1))
    y = m.node_coords()[:, 1]
    ny, c0, c1 = _analytic(wall)
    neumann = np.isclose(y, Y1) if wall == "a" else np.isclose(y, Y0)
    dirichlet = np.isclose(y, Y0) if wall == "a" else np.isclose(y, Y1)
    vel = np.tile([0.0, V], (m.n_nodes, 1))
    T = np.full(m.n_nodes, TD)
    flux = surface_term(m.axes[:2], 1, neumann[:, None], lambda p: [ny * PHI], 2)
    if method == "supg":
        kq, sq = np.full((m.n_el, 9), K), np.full((m.n_el, 9), H)
        dt = advdiff.max_dt(m, vel, kq)
        Tdot = np.zeros(m.n_nodes)
    else:
        kq, sq = np.full((m.n_el, 25), K), np.full((m.n_el, 25), H)
        dt = 5.0 * slcn.max_dt(m, vel, np.full(m.n_nodes, K))
    bcval = T.copy()
    er, its = 1.0, 0
    while er > 1e-5 and its < 2000:
        old = T.copy()
        if method == "supg":
            T, Tdot = advdiff.step(m, dt, vel, kq, sq, dirichlet, bcval, None, T, Tdot, flux=flux)
        else:
            T, _ = slcn.step(m, dt, vel, kq, sq, dirichlet, T, flux=dt * flux)
        er = np.linalg.norm(old - T) / np.linalg.norm(old)
        its += 1
    assert its < 2000
    assert _percent_error(m, T, c0, c1) < 1.0
