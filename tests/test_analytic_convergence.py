"""Convergence rates against the analytic solutions, as the reference's
convergence notebook checks them (docs/test/Analytic Soln Convergence
Tests.ipynb): relative L2 errors at resolutions 8, 16, 32 (3D: 4, 6, 8) on
Q1/dQ0 and Q2/dPc1, fitted slope within 20 % of order + 1 for velocity and of
order for pressure.  The discretisation is the oracle's (element terms of
oracle/uwo.c, direct solve of tests/oracle_system.py), the one the GPU
operators are held to at 1e-10 by the parity tests; the fields, boundary
conditions and viscosity laws are uw.function.analytic's (CPU).

The notebook's default set is A, Cx, Kx and NL; B, C, DA, DB2d, DB3d, Kz and
M are its long set.  DB3d runs on Q2/dPc1 only: with velocity fixed on every
wall of a 3D Q1/dQ0 mesh the pressure null space has dimension 3N-1, beyond
the constant and checkerboard modes any solver removes.
"""
import numpy as np
import pytest

from tests import analytic_convergence as ac
from underworld2_gb300 import function as fn

CASES = [("SolA", 1), ("SolA", 2), ("SolCx", 1), ("SolCx", 2), ("SolKx", 1), ("SolKx", 2),
         ("SolNL", 1), ("SolNL", 2), ("SolB", 1), ("SolB", 2), ("SolC", 1), ("SolC", 2),
         ("SolDA", 1), ("SolDA", 2), ("SolDB2d", 1), ("SolDB2d", 2), ("SolKz", 1), ("SolKz", 2),
         ("SolM", 1), ("SolM", 2), ("SolDB3d", 2)]


@pytest.mark.parametrize("name,order", CASES, ids=["%s-Q%d" % c for c in CASES])
def test_convergence_rate(name, order):
    sol = getattr(fn.analytic, name)()
    res = (8, 16, 32) if sol.dim == 2 else (4, 6, 8)
    v, p, (ev, ep) = ac.rates(sol, order, res)
    assert np.isclose(v, order + 1, rtol=0.2), "velocity slope %.3f (errors %s)" % (v, ev)
    assert np.isclose(p, order, rtol=0.2), "pressure slope %.3f (errors %s)" % (p, ep)
    assert ev[-1] < 0.05 and ep[-1] < 0.2


def test_solcx_vrms_known_answer():
    """docs/examples/10_Analytic_Solutions.ipynb checks the standard SolCx case
    (n_z = 1, eta_B = 1e5, Q2/dPc1, 32 x 32) for v_rms = 0.005578279626793198
    within 1e-7 relative."""
    sol = fn.analytic.SolCx(n_z=1, eta_B=100000.0)
    m, u, p = ac.solve(sol, 2, 32)
    rule = ac._Rule(m, 5)
    wq = np.tile(rule.w * rule.det, m.n_el)
    uq = np.einsum("qn,eni->eqi", rule.N, u.reshape(-1, 2)[rule.nodes]).reshape(-1, 2)
    vrms = np.sqrt(wq @ (uq ** 2).sum(1) / wq.sum())
    assert np.isclose(vrms, 0.005578279626793198, rtol=1e-7), vrms
