"""The SwarmAdvector docstring known answer (P/systems/_timeintegration.py:132-148):
one particle at (0.2, -0.2) on a 9 x 9 Q1 mesh over [-1, 1]^2, uniform velocity
(1, 1), one RK2 step at get_max_dt() lands at (0.27856742, -0.12143258).  The
oracle restates both parts: the time-step bound 0.5 x minimum node separation /
maximum speed (SwarmAdvector.c:370-387) and the RK2 step (TimeIntegrand.c:249-319).
The GPU path is held to the oracle's RK2 and max-dt by the GPU tests."""
import numpy as np

import oracle


def test_swarm_advector_docstring_step():
    m = oracle.Mesh(2, 1, (9, 9), (-1.0, -1.0), (1.0, 1.0))
    vel = np.ones((m.n_nodes, 2))
    dt = 0.5 * m.min_sep() / np.sqrt((vel ** 2).sum(1)).max()
    x, counts = m.rk2(vel, dt, np.array([[0.2, -0.2]]))
    np.testing.assert_allclose(x[0], [0.27856742, -0.12143258], rtol=1e-4)
    assert counts.tolist() == [0, 0]
