"""Known answers of the reference's extended-Boussinesq convection test
(docs/test/14_Convection_EBA.ipynb), restated on the oracle (CPU).

A 64 x 64 Q1/dQ0 unit box, Ra = 1e4, dissipation number Di = 0.5, unit
viscosity and diffusivity; T = 1 - y + 0.1 cos(pi x) sin(pi y) clipped to
[0, 1], with T = 1 on the bottom and 0 on the top; free-slip walls.  Each of
the 31 steps solves Stokes (buoyancy Ra T z on the 3 x 3 Gauss swarm), records
v_rms, Nu and the relative velocity change, then takes one SUPG step at
get_max_dt() with the source Di/Ra * 2 eta 2 II(e)^2 - Di v_y T evaluated at the
SUPG Gauss points from the current velocity and temperature (II the second
invariant of the strain rate).  Oracle pieces: tests/oracle_system.py (Stokes),
oracle/advdiff.py (SUPG).

The notebook's saved output is the reference's own run; its step 0 and step 10
lines are reproduced character for character; at steps 20 and 30 v_rms and Nu
lie within the printed rounding widened by 1e-4 relative and the two relative
changes within it widened by 5e-6 (the reference's Stokes solves are iterative
at a 1e-5 outer tolerance); its final "velocity relative tolerance"
line holds, and so does its check that the volume integrals of viscous
dissipation and adiabatic heating agree within 2 %.
"""
import numpy as np

import oracle
from oracle import advdiff
from tests import analytic_convergence as ac
from tests import oracle_system as osys

REF = {0: (17.899, 1.000, 2.000e+00, 1.000e+00), 10: (21.672, 1.059, 6.079e-03, 2.010e-02),
       20: (26.347, 1.137, 8.114e-03, 1.939e-02), 30: (31.759, 1.252, 1.083e-02, 1.838e-02)}
FMT = "steps = {0:6d}; v_rms = {1:.3f}; Nu = {2:.3f}; Rel change = {3:.3e} vChange = {4:.3e}"


def test_eba_convection_thirty_steps():
    res, Di, Ra = 64, 0.5, 1.0e4
    m = oracle.Mesh(2, 1, (res, res), (0.0, 0.0), (1.0, 1.0))
    X = m.node_coords()[:, :2]
    T = np.clip(1.0 - X[:, 1] + 0.1 * np.cos(np.pi * X[:, 0]) * np.sin(np.pi * X[:, 1]), 0.0, 1.0)
    bot, top = np.isclose(X[:, 1], 0.0), np.isclose(X[:, 1], 1.0)
    T[bot], T[top] = 1.0, 0.0
    mask = np.zeros(m.n_nodes * 2, np.uint8)
    for d in range(2):
        mask[np.flatnonzero(np.isclose(X[:, d], 0.0) | np.isclose(X[:, d], 1.0)) * 2 + d] = 1
    zero = np.zeros(m.n_nodes * 2)
    g = ac._Rule(m, 3)
    nq = len(g.w)
    pts = [(e * nq + np.arange(nq), g.xi, g.w) for e in range(m.n_el)]
    wq = np.tile(g.w * g.det, m.n_el)
    kq = np.ones((m.n_el, 9))
    h = 1.0 / res

    def nusselt(Tn):
        Tg = Tn.reshape(res + 1, res + 1)
        dTdz = (Tg[-1] - Tg[-2]) / h
        return -np.sum(0.5 * (dTdz[1:] + dTdz[:-1]) * h) / np.sum(0.5 * (Tg[0, 1:] + Tg[0, :-1]) * h)

    def heating(u, Tn):
        """(Di/Ra viscous dissipation, Di v_y T) at the Gauss points."""
        U = u.reshape(-1, 2)[g.nodes]
        grad = np.einsum("qdn,eni->eqid", g.dN, U)
        sr = 0.5 * (grad + np.swapaxes(grad, -1, -2))
        vd = 2.0 * 2.0 * 0.5 * np.einsum("eqij,eqij->eq", sr, sr)
        vy = np.einsum("qn,en->eq", g.N, U[..., 1])
        return Di / Ra * vd, Di * vy * np.einsum("qn,en->eq", g.N, Tn[g.nodes])

    u, Tdot = np.zeros(m.n_nodes * 2), np.zeros(m.n_nodes)
    step, nu_last, rerr, got = 0, -1.0, 1.0, {}
    while step <= 30 and rerr > 1e-8:
        v_old = u.copy()
        body = np.zeros((m.n_el * nq, 2))
        body[:, 1] = Ra * np.einsum("qn,en->eq", g.N, T[g.nodes]).ravel()
        u, _ = osys.solve(osys.assemble(m, pts, np.ones(m.n_el * nq), body, mask, zero), m.n_nodes * 2)
        mag = np.linalg.norm(v_old)
        rerr = np.linalg.norm(v_old - u) / mag if mag > 1e-8 else 1.0
        uq = np.einsum("qn,eni->eqi", g.N, u.reshape(-1, 2)[g.nodes]).reshape(-1, 2)
        vrms = np.sqrt(wq @ (uq ** 2).sum(1) / wq.sum())
        nu = nusselt(T)
        if step in REF:
            got[step] = (vrms, nu, abs((nu - nu_last) / nu), rerr)
        nu_last = nu
        U = u.reshape(-1, 2)
        dt = advdiff.max_dt(m, U, kq)
        vd, ad = heating(u, T)
        T, Tdot = advdiff.step(m, dt, U, kq, vd - ad, bot | top, T.copy(), None, T, Tdot)
        step += 1
    for s in (0, 10):
        assert FMT.format(s, *got[s]) == FMT.format(s, *REF[s])
    for s in (20, 30):
        vrms, nu, rel, vch = got[s]
        r_vrms, r_nu, r_rel, r_vch = REF[s]
        assert abs(vrms - r_vrms) <= 0.5e-3 + 1e-4 * r_vrms, (s, vrms)
        assert abs(nu - r_nu) <= 0.5e-3 + 1e-4 * r_nu, (s, nu)
        # differences of successive values: the solver differences enter unscaled
        for val, ref in ((rel, r_rel), (vch, r_vch)):
            assert abs(val - ref) <= 0.5e-3 * 10.0 ** np.floor(np.log10(ref)) + 5e-6, (s, val, ref)
    assert "{:.3f}".format(rerr) == "0.018"
    vd, ad = heating(u, T)
    assert np.isclose(wq @ vd.ravel(), wq @ ad.ravel(), rtol=2e-2)
