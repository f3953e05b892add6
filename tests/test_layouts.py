"""Space-filler (Sobol) and Gauss particle layouts (P/swarm/layouts.py:53-184,
L/StgFEM/Utils/src/MeshParticleLayout.c:194-230, L/StgDomain/Utils/src/
SobolGenerator.c, L/StgFEM/Discretisation/src/IrregularMeshGaussLayout.c:143-177):
the reference's docstring known answers, the closed-form Sobol values against
the generator's sequential recurrence, the vectorised skip logic against a
particle-by-particle replay, and local-to-global coordinates bit-identical with
the oracle's FeMesh_CoordLocalToGlobal."""
import numpy as np
import pytest

import oracle
import underworld2_gb300 as uw
from underworld2_gb300 import _core
from underworld2_gb300 import swarm as S


class _SeqSobol:
    """SobolGenerator_GetNextNumber as the reference iterates it: the next value
    XORs in the direction number of the rightmost zero bit of the count."""

    def __init__(self, axis):
        self.v = S._sobol_direction_numbers(axis)
        self.count = 0
        self.word = 0

    def next(self):
        c = 0
        while (self.count >> c) & 1:
            c += 1
        self.count += 1
        self.word ^= self.v[c] << (30 - c - 1)
        return self.word / float(1 << 30)


def test_docstring_known_answers():
    m = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (1, 1), (0.0, 0.0), (1.0, 1.0))
    x, _ = S._space_filler_positions(m, 4, _core.rng_seed(13))
    np.testing.assert_array_equal(x, [[0.5, 0.5], [0.25, 0.75], [0.75, 0.25], [0.375, 0.625]])
    m = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (1, 1), (-1.0, -1.0), (1.0, 1.0))
    g, per = S._gauss_positions(m, 2)
    assert per == 4
    np.testing.assert_allclose(g, [[-0.57735027, -0.57735027], [0.57735027, -0.57735027],
                                   [-0.57735027, 0.57735027], [0.57735027, 0.57735027]], atol=5e-9)


def test_layout_validation():
    m = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (2, 2), (0.0, 0.0), (1.0, 1.0))
    sw = uw.swarm.Swarm(m)
    with pytest.raises(TypeError):
        uw.swarm.layouts.PerCellSpaceFillerLayout(sw, particlesPerCell=2.0)
    with pytest.raises(ValueError):
        uw.swarm.layouts.PerCellSpaceFillerLayout(sw, particlesPerCell=0)
    with pytest.raises(ValueError):
        uw.swarm.layouts.PerCellGaussLayout(sw, gaussPointCount=6)
    with pytest.raises(TypeError):
        uw.swarm.layouts.PerCellGaussLayout(sw, gaussPointCount="2")


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_sobol_closed_form_matches_recurrence(axis):
    seq = _SeqSobol(axis)
    ref = np.array([seq.next() for _ in range(5000)])
    got = S._sobol(axis, np.arange(1, 5001, dtype=np.uint64))
    np.testing.assert_array_equal(got, ref)
    # a (0, k, 1)-net: with the initial zero, the first 2^k values fill every
    # dyadic interval of width 2^-k once
    k = 10
    cells = np.floor(np.concatenate([[0.0], got[: (1 << k) - 1]]) * (1 << k)).astype(int)
    assert sorted(cells.tolist()) == list(range(1 << k))


def test_park_miller_jump_ahead():
    state = _core.rng_seed(13)
    st, last = S._pm_draws(state, 3000)
    s, seq = state, []
    for _ in range(3000):
        s = (16807 * s) % 2147483647
        seq.append(s)
    assert st.tolist() == seq and last == seq[-1]


@pytest.mark.parametrize("et,res,ppc", [("Q1/dQ0", (3, 2), 7), ("Q2/dPc1", (2, 3), 9), ("Q1/dQ0", (2, 2, 2), 5),
                                        ("Q2/dPc1", (2, 1, 2), 6)])
def test_space_filler_matches_sequential_replay(et, res, ppc):
    """Vectorised positions (jump-ahead draws, prefix-summed skips, closed-form
    Sobol values) equal a particle-by-particle replay of the reference loop,
    with the oracle's local-to-global mapping; chunking does not matter."""
    dim = len(res)
    lo, hi = (0.25, -1.0, 0.5)[:dim], (1.5, 2.0, 1.75)[:dim]
    m = uw.mesh.FeMesh_Cartesian(et, res, lo, hi)
    om = oracle.Mesh(dim, m._order, res, lo, hi, porder=m._porder)
    state0 = _core.rng_seed(13)
    x, state = S._space_filler_positions(m, ppc, state0)
    x_chunked, state_c = S._space_filler_positions(m, ppc, state0, chunk=5)
    np.testing.assert_array_equal(x, x_chunked)
    assert state == state_c
    gens = [_SeqSobol(d) for d in range(dim)]
    s, skips = state0, 0
    for e in range(m.elementsGlobal):
        for q in range(ppc):
            s = (16807 * s) % 2147483647
            r = (1.0 - 0.0) * s / 2147483647.0 + 0.0
            xi = np.zeros(dim)
            for d in range(dim):
                if r > 0.9:
                    gens[d].next()
                xi[d] = (1.0 - -1.0) * gens[d].next() + -1.0
            skips += r > 0.9
            np.testing.assert_array_equal(x[e * ppc + q], om.local_to_global(e, xi))
    assert state == s and skips > 0


@pytest.mark.parametrize("et,res", [("Q1/dQ0", (3, 2)), ("Q2/dPc1", (2, 2)), ("Q1/dQ0", (2, 2, 3)),
                                    ("Q2/dPc1", (2, 2, 2))])
def test_local_to_global_bit_exact(et, res):
    dim = len(res)
    lo, hi = (-0.3, 0.1, 2.0)[:dim], (0.7, 1.9, 2.45)[:dim]
    m = uw.mesh.FeMesh_Cartesian(et, res, lo, hi)
    om = oracle.Mesh(dim, m._order, res, lo, hi, porder=m._porder)
    rng = np.random.default_rng(5)
    el = rng.integers(0, m.elementsGlobal, 200)
    xi = rng.uniform(-1.0, 1.0, (200, dim))
    got = S._local_to_global(m, el, xi)
    for i in range(200):
        np.testing.assert_array_equal(got[i], om.local_to_global(int(el[i]), xi[i]))
    g, per = S._gauss_positions(m, 3)
    assert g.shape == (m.elementsGlobal * 3 ** dim, dim)
