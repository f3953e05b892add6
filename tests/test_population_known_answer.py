"""Known answers of the reference's population-control test
(docs/test/population_control_test.ipynb), through the oracle.

The default mesh (2D 4 x 4 Q1 on the unit square) with PerCellGaussLayout(4):
16 particles per cell at the 4 x 4 Gauss points.  PCDVC with
* deleteThreshold 1.0, maxDeletions 15, no splits      -> 16 particles;
* deleteThreshold 0.07, maxDeletions 150, no splits    -> 64;
* splitThreshold 0, maxSplits 9999, no deletions        -> 512;
* splitThreshold 0.07, maxSplits 9999, no deletions     -> 320.
The aggressive case of the same notebook (640 particles) is not built.
The GPU population control is checked against the same oracle in
tests/test_population.py.
"""
import numpy as np
import pytest

import oracle
from oracle import population

PPC_AXIS = 4


def _gauss_swarm():
    m = oracle.Mesh(2, 1, (4, 4), (0.0, 0.0), (1.0, 1.0))
    g, _ = np.polynomial.legendre.leggauss(PPC_AXIS)
    loc = np.array([[gx, gy] for gy in g for gx in g])
    x = np.concatenate([[m.local_to_global(e, p) for p in loc] for e in range(m.n_el)])
    ppc = len(loc)
    tbl, cnt, owner = m.initial_tables(ppc, 64)
    xi, w = m.pic_map(x, tbl, cnt)
    cells = [list(tbl[e, : cnt[e]]) for e in range(m.n_el)]
    ref = population.RefSwarm(x, owner, cells, {"id": np.arange(len(x))[:, None]}, m.n_el)
    return m, ref, w, xi


@pytest.mark.parametrize("delete_t,split_t,max_del,max_split,expected", [
    (1.0, 1.0, 15, 0, 16),
    (0.07, 1.0, 150, 0, 64),
    (0.0, 0.0, 0, 9999, 512),
    (0.0, 0.07, 0, 9999, 320),
])
def test_population_counts(delete_t, split_t, max_del, max_split, expected):
    m, ref, w, xi = _gauss_swarm()
    assert ref.n == 256
    population.pcdvc(m, ref, w, xi, "id", split_t, delete_t, max_split, max_del)
    assert ref.n == expected
