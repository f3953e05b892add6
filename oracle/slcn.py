"""CPU restatement of the reference's SLCN advection-diffusion step (TEST
INFRASTRUCTURE: the checker of libuwg's uwg_slcn_phistar / uwg_slcn_solve,
never the product).

* Departure values: ``Mesh.slcn_phistar`` (oracle/uwo.c, bit-exact restatement
  of SemiLagrangianIntegrator_SolveNew,
  L/StgFEM/Utils/src/SemiLagrangianIntegrator.c:600-653).
* Crank-Nicolson system of _SLCN_AdvectionDiffusion
  (P/systems/_advectiondiffusion.py:211-259), assembled here point by point on
  the 5-point Gauss swarm the reference creates (:209):
    K_ab = sum_q w_q detJ (N_a N_b + 0.5 dt kappa_q dN_a . dN_b)
    f_a  = sum_q w_q detJ (N_a (phi*(q) + dt S_q) - 0.5 dt kappa_q dN_a . dphi*(q))
  with Dirichlet nodes removed from the numbering and their values moved to
  the right-hand side, then solved directly (scipy).  The reference solves the
  same system with a PETSc Krylov method to its default tolerance.
* Time step (get_max_dt, :777-823): min(dx / v_max, dx^2 / kappa_max) with v_max
  and kappa_max over the mesh nodes and dx the minimum node separation.
"""
import ctypes

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def gauss5():
    """5-point Gauss-Legendre rule, ascending abscissae (closed forms)."""
    a = np.sqrt(5.0 - 2.0 * np.sqrt(10.0 / 7.0)) / 3.0
    b = np.sqrt(5.0 + 2.0 * np.sqrt(10.0 / 7.0)) / 3.0
    wa = (322.0 + 13.0 * np.sqrt(70.0)) / 900.0
    wb = (322.0 - 13.0 * np.sqrt(70.0)) / 900.0
    return np.array([-b, -a, 0.0, a, b]), np.array([wb, wa, 128.0 / 225.0, wa, wb])


def gauss_points(dim):
    """Local coordinates and weights of the 5^dim points, x fastest."""
    x, w = gauss5()
    if dim == 2:
        return (np.array([[x[i], x[j]] for j in range(5) for i in range(5)]),
                np.array([w[i] * w[j] for j in range(5) for i in range(5)]))
    return (np.array([[x[i], x[j], x[k]] for k in range(5) for j in range(5) for i in range(5)]),
            np.array([w[i] * w[j] * w[k] for k in range(5) for j in range(5) for i in range(5)]))


def _elem_index(m, e):
    return [e % m.res[0], (e // m.res[0]) % m.res[1]] + ([e // (m.res[0] * m.res[1])] if m.dim == 3 else [])


def gauss_coords(m):
    """Global coordinates of the Gauss points of every element: [n_el, 5^dim, dim]."""
    xi, _ = gauss_points(m.dim)
    out = np.zeros((m.n_el, len(xi), m.dim))
    for e in range(m.n_el):
        idx = _elem_index(m, e)
        for d in range(m.dim):
            a0, a1 = m.axes[d][idx[d]], m.axes[d][idx[d] + 1]
            out[e, :, d] = a0 + 0.5 * (xi[:, d] + 1.0) * (a1 - a0)
    return out


def _shapes(m):
    xi, w = gauss_points(m.dim)
    N = np.zeros((len(w), m.nen))
    dN = np.zeros((len(w), m.dim, m.nen))
    for q in range(len(w)):
        n = np.zeros(27)
        g = np.zeros((3, 27))
        m.L.uwo_shape(m.dim, 1, ctypes.c_void_p(np.ascontiguousarray(xi[q]).ctypes.data),
                      ctypes.c_void_p(n.ctypes.data), ctypes.c_void_p(g.ctypes.data))
        N[q] = n[: m.nen]
        dN[q] = g[: m.dim, : m.nen]
    return N, dN, w


def system(m, dt, kappa_q, source_q, phistar):
    """Global (M + dt/2 D) and the right-hand side before Dirichlet elimination
    (the point loop of every element, vectorised over the elements)."""
    from oracle.advdiff import elements
    N, dN, w = _shapes(m)
    nodes, h = elements(m)
    ne, nen = m.n_el, m.nen
    detJ = np.prod(0.5 * h, axis=1)
    ps = phistar[nodes]
    Ke = np.zeros((ne, nen, nen))
    fe = np.zeros((ne, nen))
    for q in range(len(w)):
        G = dN[q][None] * (2.0 / h)[:, :, None]                     # [ne, dim, nen]
        fac = w[q] * detJ
        kq = kappa_q[:, q]
        Ke += fac[:, None, None] * (np.outer(N[q], N[q])[None] + 0.5 * dt * kq[:, None, None]
                                    * np.einsum("eda,edb->eab", G, G))
        rhs = ps @ N[q] + (dt * source_q[:, q] if source_q is not None else 0.0)
        Gps = np.einsum("eda,ea->ed", G, ps)
        fe += fac[:, None] * (N[q][None, :] * rhs[:, None] - 0.5 * dt * kq[:, None] * np.einsum("eda,ed->ea", G, Gps))
    rows = np.repeat(nodes, nen, axis=1).ravel()
    cols = np.tile(nodes, (1, nen)).ravel()
    K = sp.csr_matrix((Ke.ravel(), (rows, cols)), shape=(m.n_nodes, m.n_nodes))
    f = np.zeros(m.n_nodes)
    np.add.at(f, nodes.ravel(), fe.ravel())
    return K, f


def solve(m, dt, kappa_q, source_q, bc, phistar, phi, flux=None):
    """Solution of the Crank-Nicolson system; Dirichlet nodes keep phi's values.
    flux [n_nodes] or None: dt times the NeumannCondition surface term, added to the
    right-hand side (P/systems/_advectiondiffusion.py:237-248)."""
    K, f = system(m, dt, kappa_q, source_q, phistar)
    if flux is not None:
        f = f + flux
    bc = bc.astype(bool)
    free = ~bc
    out = phi.astype(np.float64).copy()
    rhs = f[free] - K[free][:, bc] @ out[bc]
    out[free] = spla.spsolve(K[free][:, free].tocsc(), rhs)
    return out


def step(m, dt, vel, kappa_q, source_q, bc, phi, flux=None):
    phistar = m.slcn_phistar(vel, phi, dt)
    return solve(m, dt, kappa_q, source_q, bc, phistar, phi, flux), phistar


def max_dt(m, vel, kappa_nodes):
    dx = m.min_sep()
    vmax = float(np.sqrt(np.max(np.sum(np.asarray(vel) ** 2, axis=1))))
    kmax = float(np.max(kappa_nodes))
    return min(dx / vmax, dx * dx / kmax)
