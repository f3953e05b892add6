"""The reference's Stokes sinker example (docs/examples/04_StokesSinker.ipynb),
restated on the oracle (CPU): the whole particle-in-cell path over 10 steps.

A 64 x 64 Q1/dQ0 mesh on [-1, 1] x [0, 1], free-slip walls, PerCellSpaceFiller
layout with 20 particles per cell (seed 13; positions from the package's host
layout code, which tests/test_layouts.py holds to a particle-by-particle replay
of the reference's loop), a dense sphere (radius 0.1 at (0, 0.7): viscosity 10,
density 10; elsewhere 1 and 1), body force -density z.  Each step: DVC weights
of the particles (oracle/uwo.c), PIC assembly and a direct solve
(tests/oracle_system.py), v_rms, the tracer height, then the advector's time
step 0.5 min-separation / max |v|, RK2 of the particles and of the tracer
(initially at (0, 0.6)) and the owner update.

The notebook's saved output is the reference's own run; its
"step = ...; time = ...; v_rms = ...; height = ..." lines are reproduced
character for character (4 significant digits), as are its final position line
and its v_rms check (1.0135e-2 within 1e-3).  Its pressure offsets are not
compared: they carry the arbitrary constant of its iterative pressure solve.
"""
import numpy as np

import oracle
from tests import analytic_convergence as ac
from tests import oracle_system as osys
import underworld2_gb300 as uw
from underworld2_gb300 import _core
from underworld2_gb300 import swarm as S

REFERENCE_LINES = """\
step =      0; time = 0.000e+00; v_rms = 9.022e-03; height = 6.000e-01
step =      1; time = 2.996e-01; v_rms = 9.164e-03; height = 5.925e-01
step =      2; time = 5.948e-01; v_rms = 9.316e-03; height = 5.849e-01
step =      3; time = 8.859e-01; v_rms = 9.454e-03; height = 5.774e-01
step =      4; time = 1.173e+00; v_rms = 9.571e-03; height = 5.698e-01
step =      5; time = 1.457e+00; v_rms = 9.696e-03; height = 5.623e-01
step =      6; time = 1.738e+00; v_rms = 9.797e-03; height = 5.548e-01
step =      7; time = 2.017e+00; v_rms = 9.921e-03; height = 5.472e-01
step =      8; time = 2.292e+00; v_rms = 1.001e-02; height = 5.397e-01
step =      9; time = 2.566e+00; v_rms = 1.013e-02; height = 5.321e-01"""


def test_stokes_sinker_ten_steps():
    res, ppc = 64, 20
    m = oracle.Mesh(2, 1, (res, res), (-1.0, 0.0), (1.0, 1.0))
    layout_mesh = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (res, res), (-1.0, 0.0), (1.0, 1.0))
    x, _ = S._space_filler_positions(layout_mesh, ppc, _core.rng_seed(13))
    x = np.ascontiguousarray(x)
    c = x - np.array([0.0, 0.7])
    heavy = (c * c).sum(1) < 0.1 ** 2
    eta_p = np.where(heavy, 10.0, 1.0)
    body_p = np.zeros((len(x), 2))
    body_p[:, 1] = -np.where(heavy, 10.0, 1.0)
    tbl, cnt, owner = m.initial_tables(ppc, 64)
    X = m.node_coords()[:, :2]
    mask = np.zeros(m.n_nodes * 2, np.uint8)
    for d in range(2):
        mask[np.flatnonzero(np.isclose(X[:, d], m.minc[d]) | np.isclose(X[:, d], m.maxc[d])) * 2 + d] = 1
    zero = np.zeros(m.n_nodes * 2)
    rule = ac._Rule(m, 3)
    wq = np.tile(rule.w * rule.det, m.n_el)
    tracer = np.array([[0.0, 0.6]])
    t, lines, heights = 0.0, [], []
    for step in range(10):
        xi, w = m.pic_map(x, tbl, cnt)
        sysd = osys.assemble(m, osys.pic_points_by_element(tbl, cnt, xi, w), eta_p, body_p, mask, zero)
        u, _ = osys.solve(sysd, m.n_nodes * 2)
        uq = np.einsum("qn,eni->eqi", rule.N, u.reshape(-1, 2)[rule.nodes]).reshape(-1, 2)
        vrms = np.sqrt(wq @ (uq ** 2).sum(1) / wq.sum())
        lines.append("step = {0:6d}; time = {1:.3e}; v_rms = {2:.3e}; height = {3:.3e}"
                     .format(step, t, vrms, tracer[0, 1]))
        heights.append(tracer[0, 1])
        U = u.reshape(-1, 2)
        dt = 0.5 * m.min_sep() / np.sqrt((U ** 2).sum(1)).max()
        x, _ = m.rk2(U, dt, x)
        tracer, _ = m.rk2(U, dt, tracer)
        assert m.update_owners(x, owner, tbl, cnt) == 0
        t += dt
    assert "\n".join(lines) == REFERENCE_LINES
    assert "Final position:   t = {0:.3f}, y = {1:.3f}".format(t - dt, heights[-1]) == \
        "Final position:   t = 2.566, y = 0.532"
    assert np.isclose(vrms, 1.0135e-02, rtol=1e-3)
