"""CPU tests: the oracle pinned against the reference's own golden data and
known answers, and the CPU solver against a sparse direct solve."""
import json
import os

import numpy as np
import pytest

import oracle
from tests import oracle_system

G = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def test_layout_seed13_docstring():
    """P/swarm/layouts.py:200-213: PerCellRandomLayout(seed=13) on a 1x1 mesh."""
    m = oracle.Mesh(2, 1, (1, 1), (0.0, 0.0), (1.0, 1.0))
    x, _ = m.layout_random(4, 13)
    np.testing.assert_allclose(x, G["layout_seed13_1x1_ppc4"], atol=5e-9)


def test_rk2_docstring():
    """P/systems/_timeintegration.py:132-148: one particle, v = (1, 1), dt = max dt."""
    m = oracle.Mesh(2, 1, (9, 9), (-1.0, -1.0), (1.0, 1.0))
    vel = np.ones(m.n_nodes * 2)
    dt = 0.5 * (2.0 / 9.0) / np.sqrt(2.0)
    x, counts = m.rk2(vel, dt, np.array([G["rk2_9x9"]["start"]]))
    np.testing.assert_allclose(x[0], G["rk2_9x9"]["end"], atol=5e-9)
    assert counts.tolist() == [0, 0]


def test_owner_docstring():
    """P/swarm/_swarm.py:629-639: a particle moved to (0.1, 0.1) belongs to cell 17."""
    m = oracle.Mesh(2, 1, (16, 16), (0.0, 0.0), (1.0, 1.0))
    assert m.cell_of(np.array([G["owner_16x16"]["point"]]))[0] == G["owner_16x16"]["cell"]


@pytest.mark.parametrize("dim", [2, 3])
def test_dvc_suite(dim):
    """L/PICellerator/Weights/tests/DVCWeightsSuite.c + expected/ (10 particles, 10^d grid)."""
    s = G["dvc_suite"]
    cx, w, rounds = oracle.dvc_element(dim, s["res"], np.array(s["particles_%dd" % dim]))
    np.testing.assert_allclose(cx, s["centroids_%dd" % dim], atol=1e-6)
    np.testing.assert_allclose(w, s["weights_%dd" % dim], atol=1e-12)
    assert rounds > 1


def test_dvc_is_order_sensitive():
    """The seeding rule (later particles overwrite earlier seeds) and the
    contest rule decide the weights: reversing the particle order changes
    them, so parity needs the reference's cell-table order (planted change)."""
    # on an 8x8 grid (exact binary centres) the bisector of these two particles
    # is the column of centres x = 0.125: an exact tie at every cell of it, which
    # the first claimer keeps (strict contest, DVCWeights.c:313-365)
    p = np.array([[-0.375, 0.0625], [0.625, 0.0625]])
    _, w0, _ = oracle.dvc_element(2, 8, p)
    _, w1, _ = oracle.dvc_element(2, 8, p[::-1])
    np.testing.assert_array_equal(w0 / 0.0625, [40.0, 24.0])
    np.testing.assert_array_equal(w1 / 0.0625, [32.0, 32.0])


def test_isoviscous_stiffness_matrix():
    """L/StgFEM/Assembly/tests/expected/testIsoviscousSiffness.matrix: 2D 3x3 Q1,
    unit viscosity, no BCs; Frobenius relative error < 1e-4 in the reference's
    suite, here < 1e-14."""
    K = np.array(G["isoviscous_K"]["dense"])
    m = oracle.Mesh(2, 1, (3, 3), (0.0, 0.0), (1.0, 1.0))
    xi, wt = m.gauss_points(2)
    Kg = np.zeros_like(K)
    for e in range(m.n_el):
        Ke = m.element_K(e, xi, wt, np.ones(len(wt)))
        n = m.element_nodes(e)
        idx = np.array([[2 * a, 2 * a + 1] for a in n]).ravel()
        Kg[np.ix_(idx, idx)] += Ke
    assert np.linalg.norm(Kg - K) / np.linalg.norm(K) < 1e-14


def test_newton_local_coords_affine():
    m = oracle.Mesh(3, 1, (4, 3, 2), (0.0, -1.0, 2.0), (1.0, 2.0, 3.0))
    rng = np.random.default_rng(0)
    for _ in range(20):
        x = np.array([rng.uniform(0, 1), rng.uniform(-1, 2), rng.uniform(2, 3)])
        e = m.cell_of(x[None])[0]
        xi, its = m.global_to_local(e, x)
        assert its == 2 and np.all(np.abs(xi) <= 1.0 + 1e-12)


def test_boundary_search_rules():
    """Mesh_RegularAlgorithms_SearchElements tie rules: a point on an interior
    element face belongs to the lower element; on the max face to the last."""
    m = oracle.Mesh(2, 1, (4, 4), (0.0, 0.0), (1.0, 1.0))
    assert m.cell_of(np.array([[0.5, 0.1]]))[0] == 1
    assert m.cell_of(np.array([[1.0, 1.0]]))[0] == 15
    assert m.cell_of(np.array([[0.0, 0.0]]))[0] == 0
    assert m.cell_of(np.array([[1.0 + 1e-9, 0.5]]))[0] == 16    # outside


def _sinker(dim, res, ppc):
    m = oracle.Mesh(dim, 1, res, (0.0,) * dim, (1.0,) * dim)
    x, _ = m.layout_random(ppc, 13)
    centre = np.array([0.5, 0.6, 0.5][:dim])
    inside = np.sum((x - centre) ** 2, axis=1) < 0.01
    eta = np.where(inside, 100.0, 1.0)
    body = np.zeros_like(x)
    body[:, 1] = np.where(inside, -1.0, 0.0)
    nodes = m.node_coords()
    mask = np.zeros((m.n_nodes, dim), np.uint8)
    for d in range(dim):
        mask[:, d] = np.isclose(nodes[:, d], 0.0) | np.isclose(nodes[:, d], 1.0)
    tbl, cnt, _ = m.initial_tables(ppc, ppc)
    ip_xi, ip_w = m.pic_map(x, tbl, cnt)
    return m, x, eta, body, mask.ravel(), tbl, cnt, ip_xi, ip_w


@pytest.mark.parametrize("pc", [0, 1])
@pytest.mark.parametrize("dim,res", [(2, (16, 16)), (3, (4, 4, 4)), (3, (16, 16, 16))])
def test_cpu_solver_matches_direct(dim, res, pc):
    """The CPU solver port (the timed CPU baseline) with the Uzawa term (pc 0) and
    with weighted scaled BFBt (pc 1, the GPU library's default) against the
    direct solve."""
    if res == (16, 16, 16) and pc == 0:
        pytest.skip("the Uzawa term needs hundreds of outer iterations at 16^3")
    m, x, eta, body, mask, tbl, cnt, ip_xi, ip_w = _sinker(dim, res, 12)
    pts = oracle_system.pic_points_by_element(tbl, cnt, ip_xi, ip_w)
    sysd = oracle_system.assemble(m, pts, eta, body, mask, np.zeros(len(mask)))
    uo, po = oracle_system.solve(sysd, len(mask))
    cpu = oracle.StokesCPU(m)
    cpu.set_bc(mask)
    cpu.set_schur_pc(pc)
    off = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int32)
    lst = tbl.ravel().astype(np.int32)
    slots = lst
    cpu.assemble(off, lst, ip_xi[slots], ip_w[slots], eta, body)
    u, p, st = cpu.solve(inner_rtol=1e-11, outer_rtol=1e-10)
    assert st["rc"] == 0 and st["residual"] < 1e-8
    assert np.abs(u - uo).max() <= 1e-7 * np.abs(uo).max()
    p = p - p.mean()
    assert np.abs(p - po).max() <= 1e-7 * np.abs(po).max()
    # the operator equals the assembled K on free dofs
    v = np.random.default_rng(1).standard_normal(len(mask)) * (mask == 0)
    free = mask == 0
    y = cpu.applyK(v)
    assert np.abs(y[free] - (sysd["K"] @ v)[free]).max() <= 1e-12 * np.abs(y).max()


@pytest.mark.parametrize("dim,res,expect", [(2, (6, 6), 2), (2, (5, 4), 2), (3, (4, 4, 4), 11), (3, (6, 6, 6), 17)])
def test_q1dq0_pressure_null_space_of_closed_box(dim, res, expect):
    """With velocity fixed on every wall, the gradient of a Q1/dQ0 mesh loses
    rank: in 2D the constant and the checkerboard (the two vectors the
    reference's -remove_checkerboard_pressure_null_space removes); in 3D many
    more (3N-1 on an N^3 mesh; planar checkerboards among them), which that
    removal cannot cover."""
    m = oracle.Mesh(dim, 1, res, (0.0,) * dim, (1.0,) * dim)
    gxi, gw = m.gauss_points()
    G = np.zeros((m.n_nodes * dim, m.n_el))
    for e in range(m.n_el):
        dofs = (m.element_nodes(e)[:, None] * dim + np.arange(dim)).ravel()
        G[dofs, e] += m.element_G(e, gxi, gw)[:, 0]
    nodes = m.node_coords()
    free = np.repeat(~np.any(np.isclose(nodes, 0.0) | np.isclose(nodes, 1.0), axis=1), dim)
    s = np.linalg.svd(G[free], compute_uv=False)
    assert int(np.sum(s < 1e-10 * s.max())) == expect
