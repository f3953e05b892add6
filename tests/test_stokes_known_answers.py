"""Known answers of the reference's Stokes test and example notebooks, restated on
the oracle's discretisation (element terms of oracle/uwo.c, surface term of
oracle/surface.py, direct solve of tests/oracle_system.py) -- CPU.

* docs/test/StokesEq_PoiseuilleFlow.ipynb: channel flow driven by pressure
  tractions.  A 128 x 128 Q1/dQ0 mesh on [-1, 1] x [0, 1], viscosity 1.4,
  no-slip top and bottom, v_y = 0 on every wall, and the x traction p_a = 4 on
  the left wall and -p_b = -3 on the right wall (a NeumannCondition on the x
  component of the side walls).  The velocity on the right wall must match
  u(y) = dp/dx (y^2 - h y) / (2 eta) within 1e-4 relative (the reference's run
  printed 1.4e-5, the tolerance of its iterative solve).
* docs/test/compress.ipynb: compressible extension.  A 64 x 32 Q1/dQ0 mesh on
  [0, 2] x [0, 1], viscosity 1, 1/lambda = 1e3, v_x = -0.5 / +0.5 on the left
  / right walls and v_y = 0 on the top and bottom; the volume average of
  |div v + p / lambda| must be below 1e-6 (the reference's run printed 3.5e-15).
"""
import numpy as np

import oracle
from oracle.surface import surface_term
from tests import analytic_convergence as ac
from tests import oracle_system as osys


def test_poiseuille_flow_from_pressure_tractions():
    res, eta, pa, pb, xa, xb, h = 128, 1.4, 4.0, 3.0, -1.0, 1.0, 1.0
    m = oracle.Mesh(2, 1, (res, res), (xa, 0.0), (xb, h))
    X = m.node_coords()[:, :2]
    iw = np.isclose(X[:, 0], xa) | np.isclose(X[:, 0], xb)
    jw = np.isclose(X[:, 1], 0.0) | np.isclose(X[:, 1], h)
    mask = np.zeros(m.n_nodes * 2, np.uint8)
    mask[np.flatnonzero(jw) * 2 + 0] = 1
    mask[np.flatnonzero(iw | jw) * 2 + 1] = 1
    rule = ac._Rule(m, 3)
    nq = len(rule.w)
    pts = [(e * nq + np.arange(nq), rule.xi, rule.w) for e in range(m.n_el)]
    sysd = osys.assemble(m, pts, np.full(m.n_el * nq, eta), np.zeros((m.n_el * nq, 2)), mask,
                         np.zeros(m.n_nodes * 2))
    cond = np.zeros((m.n_nodes, 2), bool)
    cond[iw, 0] = True
    traction = surface_term(m.axes[:2], 1, cond, lambda x: [pa if x[0] < 0.0 else -pb, 0.0], 2)
    sysd["f_lift"] = sysd["f_lift"] + traction[sysd["free"]]
    u, _ = osys.solve(sysd, m.n_nodes * 2, [])          # open side walls: no pressure null space
    right = np.flatnonzero(np.isclose(X[:, 0], xb))
    y = X[right, 1]
    exact = (pb - pa) / (xb - xa) * (y ** 2 - h * y) / (2.0 * eta)
    relerr = np.linalg.norm(exact - u.reshape(-1, 2)[right, 0]) / np.linalg.norm(exact)
    assert relerr < 1e-4, relerr


def test_compressible_extension_continuity():
    m = oracle.Mesh(2, 1, (64, 32), (0.0, 0.0), (2.0, 1.0))
    X = m.node_coords()[:, :2]
    left, right = np.isclose(X[:, 0], 0.0), np.isclose(X[:, 0], 2.0)
    jw = np.isclose(X[:, 1], 0.0) | np.isclose(X[:, 1], 1.0)
    mask = np.zeros(m.n_nodes * 2, np.uint8)
    val = np.zeros(m.n_nodes * 2)
    mask[np.flatnonzero(left | right) * 2] = 1
    val[np.flatnonzero(left) * 2] = -0.5
    val[np.flatnonzero(right) * 2] = 0.5
    mask[np.flatnonzero(jw) * 2 + 1] = 1
    rule = ac._Rule(m, 3)
    nq = len(rule.w)
    pts = [(e * nq + np.arange(nq), rule.xi, rule.w) for e in range(m.n_el)]
    one_on_lambda = 1.0e3
    sysd = osys.assemble(m, pts, np.ones(m.n_el * nq), np.zeros((m.n_el * nq, 2)), mask, val,
                         lam_p=np.full(m.n_el * nq, one_on_lambda))
    u, p = osys.solve(sysd, m.n_nodes * 2)
    u[sysd["bcd"]] = val[sysd["bcd"]]
    U = u.reshape(-1, 2)[rule.nodes]                                    # [ne, nen, 2]
    grad = np.einsum("qdn,eni->eqid", rule.dN, U)
    div = grad[..., 0, 0] + grad[..., 1, 1]                             # [ne, nq]
    wq = rule.w * rule.det
    err = np.sum(np.abs(div + p[:, None] * one_on_lambda) * wq[None, :]) / (2.0 * 1.0)
    assert err < 1e-6, err


def test_convection_example_vrms():
    """docs/examples/02_Convection_Example.ipynb: a 32 x 16 Q1/dQ0 box [0, 2] x [0, 1],
    Ra = 1e4, unit viscosity and diffusivity, T = 1 - y + 0.2 cos(pi x) sin(pi y)
    clipped to [0, 1] with T = 1 / 0 on the bottom / top, free-slip walls; 20
    steps of Stokes then SUPG at get_max_dt() (oracle/advdiff.py).  The notebook
    checks the final v_rms against 8.70754e+01 with numpy's default isclose."""
    from oracle import advdiff
    m = oracle.Mesh(2, 1, (32, 16), (0.0, 0.0), (2.0, 1.0))
    X = m.node_coords()[:, :2]
    T = np.clip(1.0 - X[:, 1] + 0.2 * np.cos(np.pi * X[:, 0]) * np.sin(np.pi * X[:, 1]), 0.0, 1.0)
    bot, top = np.isclose(X[:, 1], 0.0), np.isclose(X[:, 1], 1.0)
    T[bot], T[top] = 1.0, 0.0
    mask = np.zeros(m.n_nodes * 2, np.uint8)
    mask[np.flatnonzero(np.isclose(X[:, 0], 0.0) | np.isclose(X[:, 0], 2.0)) * 2] = 1
    mask[np.flatnonzero(bot | top) * 2 + 1] = 1
    rule = ac._Rule(m, 3)
    nq = len(rule.w)
    pts = [(e * nq + np.arange(nq), rule.xi, rule.w) for e in range(m.n_el)]
    kq, Tdot = np.ones((m.n_el, 9)), np.zeros(m.n_nodes)
    for _ in range(20):
        body = np.zeros((m.n_el * nq, 2))
        body[:, 1] = 1.0e4 * np.einsum("qn,en->eq", rule.N, T[rule.nodes]).ravel()
        u, _ = osys.solve(osys.assemble(m, pts, np.ones(m.n_el * nq), body, mask, np.zeros(m.n_nodes * 2)),
                          m.n_nodes * 2)
        U = u.reshape(-1, 2)
        T, Tdot = advdiff.step(m, advdiff.max_dt(m, U, kq), U, kq, None, bot | top, T.copy(), None, T, Tdot)
    wq = np.tile(rule.w * rule.det, m.n_el)
    uq = np.einsum("qn,eni->eqi", rule.N, u.reshape(-1, 2)[rule.nodes]).reshape(-1, 2)
    assert np.isclose(np.sqrt(wq @ (uq ** 2).sum(1) / wq.sum()), 8.70754e+01)
