"""CPU restatement of the reference's SUPG advection-diffusion step (TEST
INFRASTRUCTURE: the checker of libuwg's uwg_advdiff_step, never the product).

Follows, element by element and point by point:
* the explicit predictor-multicorrector,
  L/Underworld/Utils/AdvectionDiffusion/src/Multicorrector.c:166-300
  (phi += dt (1-gamma) phidot, phidot = 0; then per iteration R = residual,
  dphidot = R / M_lumped, phi += dt gamma dphidot, phidot += dphidot);
* the SUPG residual, Residual.cpp:213-341, with the upwind diffusivity of
  Residual.cpp:416-506 and the "Exact" xi of :557-568;
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
    if abs(pe) < 1.0e-8:
        return 0.33333333333333 * pe
    if pe < -20.0:
        return -1.0 - 1.0 / pe
    if pe > 20.0:
        return 1.0 - 1.0 / pe
    return math.cosh(pe) / math.sinh(pe) - 1.0 / pe


def residual(m, vel, phi, phidot, kappa_q, source_q, bc):
    """Assembled SUPG residual and lumped mass on the free nodes."""
    dim, nen = m.dim, m.nen
    gxi, gw = gauss_points(dim)
    R = np.zeros(m.n_nodes)
    M = np.zeros(m.n_nodes)
    N0, _ = _shape(m, np.zeros(dim))
    shapes = [_shape(m, gxi[q]) for q in range(len(gw))]   # the same at every element
    for e in range(m.n_el):
        nodes = m.element_nodes(e)
        idx = [e % m.res[0], (e // m.res[0]) % m.res[1]] + ([e // (m.res[0] * m.res[1])] if dim == 3 else [])
        h = [m.axes[d][idx[d] + 1] - m.axes[d][idx[d]] for d in range(dim)]
        v = vel[nodes] if vel is not None else np.zeros((nen, dim))
        kavg = float(np.sum(kappa_q[e])) / len(gw)
        if kavg < SUPG_MIN_DIFFUSIVITY:
            kavg = SUPG_MIN_DIFFUSIVITY
        vc = N0 @ v
        up = 0.0
        for d in range(dim):
            L = abs(h[d])
            up += _upwind_xi(vc[d] * L / (2.0 * kavg)) * vc[d] * L
        up *= ISQRT15
        detJ = float(np.prod([0.5 * hd for hd in h]))
        for q in range(len(gw)):
            N, dN = shapes[q]
            GNx = dN * (2.0 / np.array(h))[:, None]
            vq = N @ v
            udotu = float(vq @ vq)
            grad = GNx @ phi[nodes]
            total = float(N @ phidot[nodes]) + float(vq @ grad)
            if source_q is not None:
                total -= source_q[e, q]
            factor = gw[q] * detJ
            if abs(up) < SUPG_MIN_DIFFUSIVITY:
                supgN = N
            else:
                with np.errstate(divide="ignore", invalid="ignore"):
                    supgN = N + (up / udotu) * (vq @ GNx)
            diff = kappa_q[e, q] * (GNx.T @ grad)
            if vel is None:
                Re = -factor * diff
            else:
                Re = -factor * (supgN * total + diff)
            Me = N * N.sum() * factor
            for a in range(nen):
                if not bc[nodes[a]]:
                    R[nodes[a]] += Re[a]
                    M[nodes[a]] += Me[a]
    return R, M


def step(m, dt, vel, kappa_q, source_q, bc, bcval, bcdot, phi, phidot, iterations=2, gamma=0.5, flux=None):
    """One predictor-multicorrector step.  flux [n_nodes] or None: the boundary-flux
    vector of NeumannCondition terms (VectorSurfaceAssemblyTerm_NA__Fn__ni on the
    residual force vector, P/systems/_advectiondiffusion.py:978-991), added to the
    residual of every correction."""
    phi = phi.copy()
    phidot = phidot.copy()
    bc = bc.astype(bool)
    phi[bc] = bcval[bc]
    phidot[bc] = 0.0 if bcdot is None else bcdot[bc]
    free = ~bc
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
