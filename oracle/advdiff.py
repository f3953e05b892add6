"""CPU restatement of the reference's SUPG advection-diffusion step (TEST
INFRASTRUCTURE: the checker of libuwg's uwg_advdiff_step, never the product).

Follows, element by element and point by point:
* the explicit predictor-multicorrector,
  L/Underworld/Utils/AdvectionDiffusion/src/Multicorrector.c:166-300
  (phi += dt (1-gamma) phidot, phidot = 0 on the solution vectors; then per
  iteration R = residual of the nodal values, dphidot = R / M_lumped,
  phi += dt gamma dphidot, phidot += dphidot; the first residual sees the
  nodal values from before the predictor, see ``step``);
* the SUPG residual, Residual.cpp:213-341, with the upwind diffusivity of
  Residual.cpp:416-506 and the doubly asymptotic xi of :580-587 (the choice
  of P/systems/sle/_assemblyterm.py:388);
* the lumped mass, LumpedMassMatrixForceTerm.c:139-172;
* the time-step bound, Timestep.c:31-117;
on Q1 meshes with the default Gauss swarm (3 points per axis).  Shape
functions come from the oracle's C restatement (uwo_shape).
"""
import ctypes
import math

import numpy as np

import oracle

SUPG_MIN_DIFFUSIVITY = 1.0e-20
ISQRT15 = 0.25819888974716112567


def gauss3():
    x = math.sqrt(0.6)
    return np.array([-x, 0.0, x]), np.array([5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0])


def gauss_points(dim):
    """Local coordinates and weights of the 3^dim Gauss points, x fastest."""
    x, w = gauss3()
    if dim == 2:
        return (np.array([[x[i], x[j]] for j in range(3) for i in range(3)]),
                np.array([w[i] * w[j] for j in range(3) for i in range(3)]))
    return (np.array([[x[i], x[j], x[k]] for k in range(3) for j in range(3) for i in range(3)]),
            np.array([w[i] * w[j] * w[k] for k in range(3) for j in range(3) for i in range(3)]))


def gauss_coords(m):
    """Global coordinates of the Gauss points of every element: [n_el, 3^dim, dim]."""
    xi, _ = gauss_points(m.dim)
    out = np.zeros((m.n_el, len(xi), m.dim))
    for e in range(m.n_el):
        idx = [e % m.res[0], (e // m.res[0]) % m.res[1]] + ([e // (m.res[0] * m.res[1])] if m.dim == 3 else [])
        for d in range(m.dim):
            a0, a1 = m.axes[d][idx[d]], m.axes[d][idx[d] + 1]
            out[e, :, d] = a0 + 0.5 * (xi[:, d] + 1.0) * (a1 - a0)
    return out


def _shape(m, xi):
    N = np.zeros(27)
    G = np.zeros((3, 27))
    m.L.uwo_shape(m.dim, 1, ctypes.c_void_p(np.ascontiguousarray(xi, np.float64).ctypes.data),
                  ctypes.c_void_p(N.ctypes.data), ctypes.c_void_p(G.ctypes.data))
    return N[: m.nen], G[: m.dim, : m.nen]


def _upwind_xi(pe):
    """The doubly asymptotic upwind parameter (Residual.cpp:580-587), elementwise:
    the reference's Python interface sets "UpwindXiFunction" to
    "DoublyAsymptoticAssumption" (P/systems/sle/_assemblyterm.py:388)."""
    pe = np.asarray(pe, dtype=np.float64)
    return np.where(pe <= -3.0, -1.0, np.where(pe <= 3.0, 0.33333333333333 * pe, 1.0))


def elements(m):
    """Node lists [n_el, nen] and edge lengths [n_el, dim] of every element of a
    regular Q1 mesh (cached on the mesh)."""
    c = getattr(m, "_q1_elements", None)
    if c is None:
        nodes = np.array([m.element_nodes(e) for e in range(m.n_el)])
        e = np.arange(m.n_el)
        idx = [e % m.res[0], (e // m.res[0]) % m.res[1]] + ([e // (m.res[0] * m.res[1])] if m.dim == 3 else [])
        h = np.stack([m.axes[d][idx[d] + 1] - m.axes[d][idx[d]] for d in range(m.dim)], 1)
        c = m._q1_elements = (nodes, h)
    return c


def residual(m, vel, phi, phidot, kappa_q, source_q, bc):
    """Assembled SUPG residual and lumped mass on the free nodes, every element at
    once (the loops of Residual.cpp:213-341 over elements and points, vectorised
    over the elements)."""
    dim, nen = m.dim, m.nen
    gxi, gw = gauss_points(dim)
    nodes, h = elements(m)
    ne = m.n_el
    N0, _ = _shape(m, np.zeros(dim))
    v = vel[nodes] if vel is not None else np.zeros((ne, nen, dim))            # [ne, nen, dim]
    kavg = np.sum(kappa_q, axis=1) / len(gw)
    kavg = np.where(kavg < SUPG_MIN_DIFFUSIVITY, SUPG_MIN_DIFFUSIVITY, kavg)
    vc = np.einsum("a,ead->ed", N0, v)
    L = np.abs(h)
    up = np.sum(_upwind_xi(vc * L / (2.0 * kavg[:, None])) * vc * L, axis=1) * ISQRT15
    plain = np.abs(up) < SUPG_MIN_DIFFUSIVITY
    detJ = np.prod(0.5 * h, axis=1)
    ph, pd = phi[nodes], phidot[nodes]
    Re = np.zeros((ne, nen))
    Me = np.zeros((ne, nen))
    for q in range(len(gw)):
        N, dN = _shape(m, gxi[q])
        GNx = dN[None] * (2.0 / h)[:, :, None]                                 # [ne, dim, nen]
        vq = np.einsum("a,ead->ed", N, v)
        udotu = np.sum(vq * vq, axis=1)
        grad = np.einsum("eda,ea->ed", GNx, ph)
        total = pd @ N + np.sum(vq * grad, axis=1)
        if source_q is not None:
            total = total - source_q[:, q]
        factor = gw[q] * detJ
        with np.errstate(divide="ignore", invalid="ignore"):
            supgN = N[None, :] + (up / udotu)[:, None] * np.einsum("ed,eda->ea", vq, GNx)
        supgN = np.where(plain[:, None], N[None, :], supgN)
        diff = kappa_q[:, q][:, None] * np.einsum("eda,ed->ea", GNx, grad)
        if vel is None:
            Re -= factor[:, None] * diff
        else:
            Re -= factor[:, None] * (supgN * total[:, None] + diff)
        Me += N[None, :] * N.sum() * factor[:, None]
    free = ~np.asarray(bc, dtype=bool)[nodes]
    R = np.zeros(m.n_nodes)
    M = np.zeros(m.n_nodes)
    np.add.at(R, nodes[free], Re[free])
    np.add.at(M, nodes[free], Me[free])
    return R, M


def step(m, dt, vel, kappa_q, source_q, bc, bcval, bcdot, phi, phidot, iterations=2, gamma=0.5, flux=None):
    """One predictor-multicorrector step.  flux [n_nodes] or None: the boundary-flux
    vector of NeumannCondition terms (VectorSurfaceAssemblyTerm_NA__Fn__ni on the
    residual force vector, P/systems/_advectiondiffusion.py:978-991), added to the
    residual of every correction.

    The order is the reference's (_AdvDiffMulticorrector_Solve, Multicorrector.c:
    166-206): Dirichlet values go onto both fields; the predictor acts on the
    solution vectors only, and the residual is assembled from the fields' nodal
    values, which take the vectors' values after each corrector.  So the first
    residual sees phi_n and phidot_n as they were before the predictor; with
    d = R / M_lumped that correction gives phi = phi_n + dt (1 - gamma) phidot_n
    + dt gamma d and phidot = d, and every later one phi += dt gamma d, phidot += d."""
    phi = phi.copy()
    phidot = phidot.copy()
    bc = bc.astype(bool)
    phi[bc] = bcval[bc]
    phidot[bc] = 0.0 if bcdot is None else bcdot[bc]
    free = ~bc
    if iterations == 0:
        phi[free] += dt * (1.0 - gamma) * phidot[free]
        phidot[free] = 0.0
    M = None
    for it in range(iterations):
        R, Mi = residual(m, vel, phi, phidot, kappa_q, source_q, bc)
        if M is None:
            M = Mi
        if flux is not None:
            R = R + flux
        d = np.zeros_like(phi)
        d[free] = R[free] / M[free]
        if it == 0:
            phi[free] = (phi[free] + dt * (1.0 - gamma) * phidot[free]) + dt * gamma * d[free]
            phidot[free] = d[free]
        else:
            phi[free] += dt * gamma * d[free]
            phidot[free] += d[free]
    return phi, phidot


def max_dt(m, vel, kappa_q, courant=0.5):
    sep = [float(np.min(np.abs(np.diff(m.axes[d])))) for d in range(m.dim)]
    minsep = min(sep)
    adv = math.inf
    if vel is not None:
        for d in range(m.dim):
            vd = vel[:, d]
            nz = vd != 0.0
            if np.any(nz):
                adv = min(adv, float(np.min(np.abs(sep[d] / vd[nz]))))
    kmax = float(np.max(kappa_q))
    diff = minsep * minsep / kmax if kmax > 0 else math.inf
    return courant * min(adv, diff)
