"""Convergence of the oracle's Stokes discretisation against the analytic
solutions of ``uw.function.analytic`` (test helper, CPU only).

Follows the reference's convergence notebook (docs/test/Analytic Soln
Convergence Tests.ipynb): a Q1/dQ0 or Q2/dPc1 mesh on the unit square, the
solution's viscosity and body force at Gauss points, its boundary conditions,
a direct solve (nonlinear solutions: a constant-viscosity solve, then Picard
iterations on the solution's viscosity law to a relative change of 1e-7),
then relative L2 errors of velocity and of mean-free pressure on a 3-point
Gauss rule, and the slope of log(error) against log(h).
"""
import ctypes

import numpy as np

import oracle
from tests import oracle_system as osys


def _shape(m, xi):
    N = np.zeros(27)
    G = np.zeros((3, 27))
    m.L.uwo_shape(m.dim, m.order, ctypes.c_void_p(np.ascontiguousarray(xi, np.float64).ctypes.data),
                  ctypes.c_void_p(N.ctypes.data), ctypes.c_void_p(G.ctypes.data))
    return N[: m.nen], G[: m.dim, : m.nen]


def _pshape(m, xi):
    M = np.zeros(4)
    m.L.uwo_pressure_shape(m.dim, m.porder, ctypes.c_void_p(np.ascontiguousarray(xi, np.float64).ctypes.data),
                           ctypes.c_void_p(M.ctypes.data))
    return M[: m.npn]


class _Rule:
    """Gauss points of every element: local coords, weights x detJ, global coords,
    shape values and global derivatives (regular mesh: diagonal Jacobian)."""

    def __init__(self, m, n):
        xi, w = m.gauss_points(n)
        h = np.array([(m.maxc[d] - m.minc[d]) / m.res[d] for d in range(m.dim)])
        self.xi, self.w = xi, w
        self.det = float(np.prod(h / 2.0))
        self.N, self.dN = [], []
        for q in range(len(xi)):
            N, G = _shape(m, xi[q])
            self.N.append(N)
            self.dN.append(G * (2.0 / h)[:, None])
        self.N, self.dN = np.array(self.N), np.array(self.dN)       # [nq, nen], [nq, dim, nen]
        self.M = np.array([_pshape(m, xi[q]) for q in range(len(xi))])   # [nq, npn]
        self.x = np.array([[m.local_to_global(e, xi[q]) for q in range(len(xi))] for e in range(m.n_el)])
        self.nodes = np.array([m.element_nodes(e) for e in range(m.n_el)])


def _node_weights_1d(c, order):
    """int N_i along an axis: trapezoid (order 1) or Simpson (order 2) weights."""
    w = np.zeros(len(c))
    for a in range(0, len(c) - 1, order):
        h = c[a + order] - c[a]
        if order == 1:
            w[a:a + 2] += 0.5 * h
        else:
            w[a:a + 3] += np.array([1.0, 4.0, 1.0]) * h / 6.0
    return w


def _wall_flux(sol, m, d, side):
    """int of the analytic normal velocity over the wall x_d = side (6-point
    Gauss per element edge/face)."""
    g, gw = np.polynomial.legendre.leggauss(6)
    others = [e for e in range(m.dim) if e != d]
    grids = []
    for e in others:
        a = m.axes[e][:: m.order]
        mid, half = 0.5 * (a[1:] + a[:-1]), 0.5 * (a[1:] - a[:-1])
        grids.append(((mid[:, None] + half[:, None] * g[None, :]).ravel(), (half[:, None] * gw[None, :]).ravel()))
    mesh_pts = np.meshgrid(*[c for c, _ in grids], indexing="ij")
    mesh_w = np.meshgrid(*[w for _, w in grids], indexing="ij")
    X = np.zeros((mesh_pts[0].size, m.dim))
    X[:, d] = side
    for i, e in enumerate(others):
        X[:, e] = mesh_pts[i].ravel()
    W = np.prod([w.ravel() for w in mesh_w], axis=0)
    return float(W @ sol.fn_velocity.evaluate(X)[:, d])


def _wall_masks(m, sol, vel_bc):
    dim = m.dim
    X = m.node_coords()[:, :dim]
    mask = np.zeros(m.n_nodes * dim, np.uint8)
    val = np.zeros(m.n_nodes * dim)
    on = [(np.isclose(X[:, d], m.minc[d]) | np.isclose(X[:, d], m.maxc[d])) for d in range(dim)]
    if getattr(sol, "fixed_walls", False):
        # every component on every wall at the analytic value, each wall's normal
        # component shifted so that its numerical flux is the analytic one
        walls = np.flatnonzero(np.any(on, axis=0))
        mask[(walls[:, None] * dim + np.arange(dim)).ravel()] = 1
        V = np.zeros((m.n_nodes, dim))
        V[walls] = vel_bc(X[walls])
        nn = [len(a) for a in m.axes[:dim]]
        idx = np.indices(nn[::-1]).reshape(dim, -1)[::-1]            # node i, j[, k] (x fastest)
        for d in range(dim):
            for side in (m.minc[d], m.maxc[d]):
                nodes = np.flatnonzero(np.isclose(X[:, d], side))
                w = np.ones(len(nodes))
                for e in range(dim):
                    if e != d:
                        w *= _node_weights_1d(m.axes[e], m.order)[idx[e, nodes]]
                V[nodes, d] -= w @ V[nodes, d] - _wall_flux(sol, m, d, side)
        val[:] = V.ravel()
    elif not sol.nonlinear:
        for d in range(dim):           # free slip: the normal component on each wall
            mask[np.flatnonzero(on[d]) * dim + d] = 1
    else:                              # x on the vertical walls, z on every wall
        iw, jw = on[0], on[0] | on[1]
        mask[np.flatnonzero(iw) * dim + 0] = 1
        mask[np.flatnonzero(jw) * dim + 1] = 1
        val[:] = vel_bc(X).ravel()
    return mask, val


def _second_invariant_dev(gu):
    """sqrt(1/2 D:D) with D the deviatoric part of the symmetric gradient: [n, d, d]."""
    d = gu.shape[-1]
    s = 0.5 * (gu + np.swapaxes(gu, -1, -2))
    s = s - np.trace(s, axis1=-2, axis2=-1)[:, None, None] * np.eye(d) / d
    return np.sqrt(0.5 * np.einsum("nij,nij->n", s, s))


def solve(sol, order, res, picard_tol=1e-7, max_picard=200):
    """Numerical velocity (nodal) and pressure (per element) for `sol`."""
    dim = sol.dim
    m = oracle.Mesh(dim, order, (res,) * dim, (0.0,) * dim, (1.0,) * dim, porder=order - 1)
    rule = _Rule(m, 3 if order == 1 else 5)
    xq = rule.x.reshape(-1, dim)
    nq = len(rule.w)
    body = sol.fn_bodyforce.evaluate(xq)
    eta = sol.fn_viscosity.evaluate(xq)[:, 0] if not sol.nonlinear else np.ones(len(xq))
    mask, val = _wall_masks(m, sol, lambda X: sol.fn_velocity.evaluate(X))
    pts = [(e * nq + np.arange(nq), rule.xi, rule.w) for e in range(m.n_el)]

    null = None
    if getattr(sol, "fixed_walls", False) and order == 1:
        null = osys.checkerboard_vectors(m.res)      # all-wall Dirichlet Q1/dQ0: constant + checkerboard

    def run(eta_q):
        sysd = osys.assemble(m, pts, eta_q, body, mask, val)
        u, p = osys.solve(sysd, m.n_nodes * dim, null)
        u[sysd["bcd"]] = val[sysd["bcd"]]
        return u, p

    u, p = run(eta)
    if sol.nonlinear:
        al2 = 2.0 / sol.r - 2.0
        for _ in range(max_picard):
            U = u.reshape(-1, 2)[rule.nodes]                         # [ne, nen, 2]
            gu = np.einsum("qdn,eni->eqid", rule.dN, U).reshape(-1, 2, 2)
            eta = 2.0 * sol.eta_0 * _second_invariant_dev(gu) ** al2
            u_new, p = run(eta)
            change = np.linalg.norm(u_new - u) / np.linalg.norm(u_new)
            u = u_new
            if change < picard_tol:
                break
        else:
            raise RuntimeError("Picard iterations did not converge")
    return m, u, p


def errors(sol, m, u, p):
    """Relative L2 errors (velocity, mean-free pressure) on 3 Gauss points per axis."""
    dim = m.dim
    rule = _Rule(m, 3)
    xq = rule.x.reshape(-1, dim)
    wq = np.tile(rule.w * rule.det, m.n_el)
    U = u.reshape(-1, dim)[rule.nodes]
    uh = np.einsum("qn,eni->eqi", rule.N, U).reshape(-1, dim)
    P = p.reshape(m.n_el, m.npn)
    ph = np.einsum("qb,eb->eq", rule.M, P).ravel()
    ua = sol.fn_velocity.evaluate(xq)
    pa = sol.fn_pressure.evaluate(xq)[:, 0]
    vol = wq.sum()
    ph = ph - (wq @ ph) / vol
    pa = pa - (wq @ pa) / vol
    ev = np.sqrt(wq @ ((ua - uh) ** 2).sum(1)) / np.sqrt(wq @ (ua ** 2).sum(1))
    ep = np.sqrt(wq @ (pa - ph) ** 2) / np.sqrt(wq @ pa ** 2)
    return ev, ep


def rates(sol, order, resolutions=(8, 16, 32)):
    """(velocity slope, pressure slope, errors) of log(error) against log(1/res)."""
    ev, ep = [], []
    for r in resolutions:
        m, u, p = solve(sol, order, r)
        a, b = errors(sol, m, u, p)
        ev.append(a)
        ep.append(b)
    lh = np.log(1.0 / np.asarray(resolutions, dtype=float))
    return np.polyfit(lh, np.log(ev), 1)[0], np.polyfit(lh, np.log(ep), 1)[0], (ev, ep)
