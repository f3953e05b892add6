"""Particle deletion and creation with the reference's swarm semantics.

CPU: the oracle's population control splits every particle once when the
split threshold is 0 (the PopulationControl docstring's doubling,
P/swarm/_population_control.py:60-68).  GPU: escaped-particle removal and
PCDVC population control through the uw-style API, compared with the oracle's
line-by-line restatement of the reference's array and cell-table edits:
coordinates, owners, cell tables and swarm-variable rows exactly equal.
"""
import numpy as np
import pytest
import torch

import oracle
from oracle import population


def _ref_swarm(m, coords, owner, tbl, cnt, data):
    cells = [list(tbl[e, : cnt[e]]) for e in range(m.n_el)]
    return population.RefSwarm(coords, owner, cells, data, m.n_el)


def test_oracle_split_everything_doubles():
    m = oracle.Mesh(2, 1, (4, 4), (0.0, 0.0), (1.0, 1.0))
    ppc = 6
    x, _ = m.layout_random(ppc, 3)
    tbl, cnt, owner = m.initial_tables(ppc, 64)
    xi, w = m.pic_map(x, tbl, cnt)
    ref = _ref_swarm(m, x, owner, tbl, cnt, {"id": np.arange(len(x))[:, None]})
    ns, nd = population.pcdvc(m, ref, w, xi, "id", 0.0, 0.0, 9999, 0)
    assert (ns, nd) == (len(x), 0) and ref.n == 2 * len(x)
    off, lst = ref.tables()
    assert sorted(lst.tolist()) == list(range(ref.n))


def _gpu_state(swarm, ids, val):
    off = swarm._off.cpu().numpy()
    lst = swarm._lst.cpu().numpy()[: off[-1]]
    return (swarm.data.copy(), swarm._owner.cpu().numpy(), off, lst, ids.data.copy(), val.data.copy())


def _check(state, ref):
    x, owner, off, lst, ids, val = state
    roff, rlst = ref.tables()
    np.testing.assert_array_equal(x, np.array(ref.x))
    np.testing.assert_array_equal(owner, np.array(ref.owner))
    np.testing.assert_array_equal(off, roff)
    np.testing.assert_array_equal(lst, rlst)
    np.testing.assert_array_equal(ids, np.array(ref.data["id"]))
    np.testing.assert_array_equal(val, np.array(ref.data["val"]))


def _setup(res, ppc, escape, seed=5):
    import underworld2_gb300 as uw
    dim = len(res)
    mesh = uw.mesh.FeMesh_Cartesian(elementRes=res, minCoord=(0.0,) * dim, maxCoord=(1.0,) * dim)
    swarm = uw.swarm.Swarm(mesh, particleEscape=escape)
    swarm.populate_using_layout(uw.swarm.layouts.PerCellRandomLayout(swarm, particlesPerCell=ppc, seed=seed))
    ids = swarm.add_variable("int", 1)
    ids.data[:, 0] = np.arange(swarm.particleLocalCount)
    val = swarm.add_variable("double", 2)
    val.data[...] = np.random.default_rng(seed).standard_normal((swarm.particleLocalCount, 2))
    m = oracle.Mesh(dim, 1, res, (0.0,) * dim, (1.0,) * dim)
    x0, _ = m.layout_random(ppc, seed)
    np.testing.assert_array_equal(swarm.data, x0)
    tbl, cnt, owner = m.initial_tables(ppc, 4 * ppc)
    return uw, mesh, swarm, ids, val, m, x0, tbl, cnt, owner


@pytest.mark.gpu
@pytest.mark.parametrize("res", [(6, 5), (3, 4, 3)])
def test_escaped_particles_removed_as_reference(gpu, res):
    uw, mesh, swarm, ids, val, m, x0, tbl, cnt, owner = _setup(res, 10, True)
    x1 = x0.copy()
    x1[:, 0] += 0.3 * x1[:, -1]          # particles near x = 1 and high up leave the mesh
    x1[::7, 1] -= 0.2                     # and some through the bottom
    data = {"id": ids.data.copy(), "val": val.data.copy()}
    with swarm.deform_swarm():
        swarm.data[...] = x1
    coords = x1.copy()
    lost = m.update_owners(coords, owner, tbl, cnt)
    assert lost > 0
    ref = _ref_swarm(m, coords, owner, tbl, cnt, data)
    ref.remove_escaped()
    assert swarm.particleLocalCount == ref.n == len(x0) - lost
    _check(_gpu_state(swarm, ids, val), ref)


@pytest.mark.gpu
def test_escape_without_flag_raises_after_removal(gpu):
    uw, mesh, swarm, ids, val, m, x0, tbl, cnt, owner = _setup((5, 5), 6, False)
    n0 = swarm.particleLocalCount
    with pytest.raises(RuntimeError):
        with swarm.deform_swarm():
            swarm.data[:3, 0] = 1.5
    assert swarm.particleLocalCount == n0 - 3


@pytest.mark.gpu
@pytest.mark.parametrize("res,ppc", [((6, 5), 12), ((3, 3, 3), 14)])
def test_population_control_matches_reference(gpu, res, ppc):
    uw, mesh, swarm, ids, val, m, x0, tbl, cnt, owner = _setup(res, ppc, False, seed=9)
    dim = len(res)
    h = 1.0 / np.array(res)
    lo = np.floor(x0 / h) * h
    x1 = x0.copy()
    cell = owner
    squeeze = (cell % 3) == 0                  # crowd these elements into a corner: large empty Voronoi cells
    x1[squeeze] = lo[squeeze] + 0.2 * (x0[squeeze] - lo[squeeze])
    twin = np.where((cell % 3) == 1)[0][::ppc]  # near-duplicates: tiny Voronoi cells
    x1[twin] = x1[twin + 1] + 1e-4 * h
    assert (m.cell_of(x1) == owner).all()   # every particle stays in its element
    data = {"id": ids.data.copy(), "val": val.data.copy()}
    with swarm.deform_swarm():
        swarm.data[...] = x1
    pc = uw.swarm.PopulationControl(swarm, deleteThreshold=0.02, splitThreshold=0.12, maxDeletions=2, maxSplits=3)
    pc.repopulate()
    xi, w = m.pic_map(x1, tbl, cnt)
    ref = _ref_swarm(m, x1, owner, tbl, cnt, data)
    ns, nd = population.pcdvc(m, ref, w, xi, "id", 0.12, 0.02, 3, 2)
    assert ns > 0 and nd > 0
    assert (pc.last["splits"], pc.last["deletions"]) == (ns, nd)
    _check(_gpu_state(swarm, ids, val), ref)
    # a second pass over the edited swarm
    pc.repopulate()
    off, lst = ref.tables()
    n_ref = ref.n
    cnt2 = np.diff(off).astype(np.int32)
    tbl2 = np.full((m.n_el, max(cnt2.max(), 1) + 8), -1, np.int32)
    for e in range(m.n_el):
        tbl2[e, : cnt2[e]] = lst[off[e]: off[e + 1]]
    xi2, w2 = m.pic_map(np.array(ref.x), tbl2, cnt2)
    ref.data["id"] = [np.array([i]) for i in range(n_ref)]
    population.pcdvc(m, ref, w2, xi2, "id", 0.12, 0.02, 3, 2)
    x, owner2, goff, glst, _, _ = _gpu_state(swarm, ids, val)
    np.testing.assert_array_equal(x, np.array(ref.x))
    np.testing.assert_array_equal(goff, ref.tables()[0])
    np.testing.assert_array_equal(glst, ref.tables()[1])
