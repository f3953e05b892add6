"""GPU parity of the PIC Stokes path against the CPU oracle (through the C ABI).

Bit-exact: particle layout, element ownership, Newton local coordinates, DVC
centroids and weights, RK2 positions, owner update and cell tables.
Tolerance: element matrices 1e-10 relative (FP64), operator applies 1e-12,
solutions 1e-7 relative to the field scale (both sides converged to 1e-10).
"""
import numpy as np
import pytest
import torch

import oracle
from tests import oracle_system

pytestmark = pytest.mark.gpu

CASES = [
    (2, (8, 8), 5),
    (2, (7, 5), 3),
    (3, (4, 4, 4), 4),
    (3, (3, 2, 5), 6),
]


def _ctx(dim, res):
    from underworld2_gb300._core import Context
    return Context(dim, res, (0.0,) * dim, (1.0,) * dim)


def _oracle_mesh(dim, res):
    return oracle.Mesh(dim, 1, res, (0.0,) * dim, (1.0,) * dim)


@pytest.mark.parametrize("dim,res,ppc", CASES)
def test_layout_locate_map_dvc_bit_exact(gpu, dim, res, ppc):
    from underworld2_gb300._core import rng_seed
    c = _ctx(dim, res)
    m = _oracle_mesh(dim, res)
    x, owner, off, lst, st = c.layout_random(ppc, rng_seed(13))
    xo, sto = m.layout_random(ppc, 13)
    assert st == sto
    np.testing.assert_array_equal(x.cpu().numpy(), xo)
    np.testing.assert_array_equal(c.locate(x).cpu().numpy(), m.cell_of(xo))
    ip_xi = c.pic_map(x, off, lst)
    tbl, cnt, _ = m.initial_tables(ppc, ppc)
    ref_xi = np.stack([m.global_to_local(e, xo[p])[0] for e in range(m.n_el) for p in tbl[e]])
    np.testing.assert_array_equal(ip_xi.cpu().numpy(), ref_xi)
    ip_w = c.dvc_weights(off, ip_xi)
    oxi, ow = m.pic_map(xo, tbl, cnt)
    slots = np.concatenate([tbl[e, : cnt[e]] for e in range(m.n_el)])
    np.testing.assert_array_equal(ip_xi.cpu().numpy(), oxi[slots])
    np.testing.assert_array_equal(ip_w.cpu().numpy(), ow[slots])


def test_dvc_golden_suite(gpu):
    """The reference's DVC suite particle sets (10 particles, 10^d grid), one element."""
    import json, os
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))["dvc_suite"]
    for dim in (2, 3):
        p = np.array(g["particles_%dd" % dim])
        c = _ctx(dim, (1,) * dim)
        off = torch.tensor([0, len(p)], dtype=torch.int32, device="cuda")
        xi = torch.tensor(p, dtype=torch.float64, device="cuda")
        w = c.dvc_weights(off, xi, res=10)
        np.testing.assert_allclose(xi.cpu().numpy(), np.array(g["centroids_%dd" % dim]), atol=1e-6)
        np.testing.assert_allclose(w.cpu().numpy(), np.array(g["weights_%dd" % dim]), atol=1e-12)
        cx, wo, _ = oracle.dvc_element(dim, 10, p)
        np.testing.assert_array_equal(xi.cpu().numpy(), cx)


def _circle_problem(dim, res, ppc):
    """Sinker: circle/sphere of radius 0.1 at (0.5, 0.6[, 0.5]), eta 100, rho 1."""
    from underworld2_gb300._core import rng_seed
    c = _ctx(dim, res)
    m = _oracle_mesh(dim, res)
    x, owner, off, lst, _ = c.layout_random(ppc, rng_seed(13))
    xo, _ = m.layout_random(ppc, 13)
    centre = np.array([0.5, 0.6, 0.5][:dim])
    inside = np.sum((xo - centre) ** 2, axis=1) < 0.1 ** 2
    eta = np.where(inside, 100.0, 1.0)
    body = np.zeros((len(xo), dim))
    body[:, 1] = np.where(inside, -1.0, 0.0)
    # free-slip walls
    nodes = m.node_coords()
    mask = np.zeros((m.n_nodes, dim), np.uint8)
    for d in range(dim):
        mask[:, d] = (np.isclose(nodes[:, d], 0.0) | np.isclose(nodes[:, d], 1.0)).astype(np.uint8)
    return c, m, (x, owner, off, lst), xo, eta, body, mask.ravel()


@pytest.mark.parametrize("dim,res,ppc", [(2, (8, 8), 20), (3, (4, 4, 4), 8)])
def test_assembly_and_operators(gpu, dim, res, ppc):
    c, m, (x, owner, off, lst), xo, eta, body, mask = _circle_problem(dim, res, ppc)
    ip_xi = c.pic_map(x, off, lst)
    ip_w = c.dvc_weights(off, ip_xi)
    c.set_bcs(torch.tensor(mask, device="cuda"))
    eta_t = torch.tensor(eta, device="cuda")
    body_t = torch.tensor(body, device="cuda")
    c.assemble(off, lst, ip_xi, ip_w, eta_t, body_t)
    tbl, cnt, _ = m.initial_tables(ppc, ppc)
    oxi, ow = m.pic_map(xo, tbl, cnt)
    pts = oracle_system.pic_points_by_element(tbl, cnt, oxi, ow)
    for e in [0, m.n_el // 2, m.n_el - 1]:
        Ke, Ge, Se = c.element_matrices(e)
        ps, xi, w = pts[e]
        Ko = m.element_K(e, xi, w, eta[ps])
        assert np.abs(Ke - Ko).max() <= 1e-10 * np.abs(Ko).max()
        gxi, gw = m.gauss_points()
        Go = m.element_G(e, gxi, gw)
        assert np.abs(Ge - Go).max() <= 1e-12 * np.abs(Go).max()
        So = m.element_S(Ko, Go)
        assert abs(Se[0, 0] - So[0, 0]) <= 1e-10 * abs(So[0, 0])
    sysd = oracle_system.assemble(m, pts, eta, body, mask, np.zeros(len(mask)))
    rng = np.random.default_rng(0)
    xv = rng.standard_normal(m.n_nodes * dim) * (mask == 0)
    y = c.apply_K(torch.tensor(xv, device="cuda")).cpu().numpy()
    yo = sysd["K"] @ xv
    free = mask == 0
    assert np.abs(y[free] - yo[free]).max() <= 1e-12 * np.abs(yo).max()
    y32 = c.apply_K(torch.tensor(xv, device="cuda", dtype=torch.float32)).cpu().numpy()
    assert np.abs(y32[free] - yo[free]).max() <= 1e-5 * np.abs(yo).max()
    pv = rng.standard_normal(m.n_el)
    yg = c.apply_G(torch.tensor(pv, device="cuda")).cpu().numpy()
    assert np.abs(yg[free] - (sysd["G"] @ pv)[free]).max() <= 1e-12 * np.abs(yg).max()
    q = c.apply_Gt(torch.tensor(xv, device="cuda")).cpu().numpy()
    assert np.abs(q - sysd["G"].T @ xv).max() <= 1e-12 * np.abs(q).max()


@pytest.mark.parametrize("mixed", [0, 1])
@pytest.mark.parametrize("dim,res,ppc", [(2, (16, 16), 20), (3, (4, 4, 4), 8)])
def test_solve_matches_direct(gpu, dim, res, ppc, mixed):
    c, m, (x, owner, off, lst), xo, eta, body, mask = _circle_problem(dim, res, ppc)
    ip_xi = c.pic_map(x, off, lst)
    ip_w = c.dvc_weights(off, ip_xi)
    c.set_bcs(torch.tensor(mask, device="cuda"))
    c.assemble(off, lst, ip_xi, ip_w, torch.tensor(eta, device="cuda"), torch.tensor(body, device="cuda"))
    u = c.zeros(m.n_nodes * dim)
    p = c.zeros(m.n_el)
    st = c.solve(u, p, mixed=mixed, rtol=1e-8, inner_rtol=1e-11, outer_rtol=1e-10)
    assert st["residual"] <= 1e-8, st
    tbl, cnt, _ = m.initial_tables(ppc, ppc)
    oxi, ow = m.pic_map(xo, tbl, cnt)
    pts = oracle_system.pic_points_by_element(tbl, cnt, oxi, ow)
    sysd = oracle_system.assemble(m, pts, eta, body, mask, np.zeros(len(mask)))
    uo, po = oracle_system.solve(sysd, m.n_nodes * dim)
    ug = u.cpu().numpy()
    pg = p.cpu().numpy()
    pg = pg - pg.mean()
    assert np.abs(ug - uo).max() <= 1e-7 * np.abs(uo).max()
    assert np.abs(pg - po).max() <= 1e-7 * np.abs(po).max()
    # advection: velocity field from the solve, one RK2 step at the reference's max dt
    vel = u.view(-1, dim)
    dt = c.max_dt(u)
    vmax = np.sqrt((uo.reshape(-1, dim) ** 2).sum(1)).max()
    assert abs(dt - 0.5 * (1.0 / max(res)) / vmax) <= 1e-6 * dt
    x_gpu = x.clone()
    fb, failed = c.rk2(x_gpu, u, dt)
    x_or, counts = m.rk2(ug, dt, xo.copy())
    assert failed == counts[0] and fb == counts[1]
    np.testing.assert_array_equal(x_gpu.cpu().numpy(), x_or)


# meshes above one block of cells (128) as well as below
@pytest.mark.parametrize("dim,res", [(2, (6, 6)), (3, (3, 3, 3)), (2, (24, 20)), (3, (8, 7, 6))])
def test_owner_update_tables(gpu, dim, res):
    """Random moves; owners and cell tables equal the sequential reference semantics."""
    from underworld2_gb300._core import rng_seed
    c = _ctx(dim, res)
    m = _oracle_mesh(dim, res)
    ppc = 6
    x, owner, off, lst, _ = c.layout_random(ppc, rng_seed(7))
    xo, _ = m.layout_random(ppc, 7)
    tbl, cnt, own_o = m.initial_tables(ppc, 64)
    rng = np.random.default_rng(3)
    for step in range(4):
        delta = rng.uniform(-0.3, 0.3, xo.shape) / max(res)
        xo = np.clip(xo + delta, 0.0, 1.0)
        if step == 2:
            xo[5] = [1.2] + [0.5] * (dim - 1)     # leaves the domain
        x = torch.tensor(xo, device="cuda")
        lost = c.update_owners(x, owner, off, lst)
        lost_o = m.update_owners(xo, own_o, tbl, cnt)
        assert lost == lost_o
        np.testing.assert_array_equal(owner.cpu().numpy(), own_o)
        offn = off.cpu().numpy()
        lstn = lst.cpu().numpy()
        for e in range(m.n_el):
            np.testing.assert_array_equal(lstn[offn[e]: offn[e + 1]], tbl[e, : cnt[e]])


def test_golden_known_answers(gpu):
    import json, os
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))
    from underworld2_gb300._core import rng_seed
    c = _ctx(2, (1, 1))
    x, *_ = c.layout_random(4, rng_seed(13))
    np.testing.assert_allclose(x.cpu().numpy(), np.array(g["layout_seed13_1x1_ppc4"]), atol=5e-9)
    from underworld2_gb300._core import Context
    c = Context(2, (9, 9), (-1.0, -1.0), (1.0, 1.0))
    vel = torch.ones(c.n_nodes * 2, dtype=torch.float64, device="cuda")
    dt = c.max_dt(vel)
    pts = torch.tensor([g["rk2_9x9"]["start"]], dtype=torch.float64, device="cuda")
    c.rk2(pts, vel, dt)
    np.testing.assert_allclose(pts.cpu().numpy()[0], g["rk2_9x9"]["end"], atol=5e-9)
    c = Context(2, (16, 16), (0.0, 0.0), (1.0, 1.0))
    own = c.locate(torch.tensor([g["owner_16x16"]["point"]], dtype=torch.float64, device="cuda"))
    assert int(own.cpu()[0]) == g["owner_16x16"]["cell"]


def test_dvc_exact_ties_follow_particle_order(gpu):
    """Exact distance ties go to the first claimer: GPU matches the oracle for
    both particle orders (8x8 grid with binary-exact cell centres)."""
    c = _ctx(2, (1, 1))
    off = torch.tensor([0, 2], dtype=torch.int32, device="cuda")
    for p in (np.array([[-0.375, 0.0625], [0.625, 0.0625]]), np.array([[0.625, 0.0625], [-0.375, 0.0625]])):
        xi = torch.tensor(p, dtype=torch.float64, device="cuda")
        w = c.dvc_weights(off, xi, res=8)
        cx, wo, _ = oracle.dvc_element(2, 8, p)
        np.testing.assert_array_equal(w.cpu().numpy(), wo)
        np.testing.assert_array_equal(xi.cpu().numpy(), cx)


@pytest.mark.parametrize("dim", [2, 3])
def test_dvc_random_many_particles(gpu, dim):
    """Crowded elements (up to 100 particles) and a 16^d grid, bit-exact."""
    rng = np.random.default_rng(11)
    counts = [1, 2, 7, 33, 64, 100]
    pts = [rng.uniform(-1, 1, (n, dim)) for n in counts]
    c = _ctx(dim, (len(counts),) + (1,) * (dim - 1))
    off = torch.tensor(np.concatenate([[0], np.cumsum(counts)]), dtype=torch.int32, device="cuda")
    xi = torch.tensor(np.concatenate(pts), dtype=torch.float64, device="cuda")
    w = c.dvc_weights(off, xi, res=16 if dim == 2 else 12)
    for k, p in enumerate(pts):
        cx, wo, _ = oracle.dvc_element(dim, 16 if dim == 2 else 12, p)
        s = slice(int(off[k]), int(off[k + 1]))
        np.testing.assert_array_equal(w.cpu().numpy()[s], wo)
        np.testing.assert_array_equal(xi.cpu().numpy()[s], cx)


def test_initial_guess(gpu):
    """zero_guess = 0 starts FGMRES (and the back-solve) from the given p (u):
    restarting from a converged solution takes no outer iteration, and from a
    perturbed one fewer than from zero, with the same result."""
    c, m, (x, owner, off, lst), xo, eta, body, mask = _circle_problem(2, (16, 16), 20)
    ip_xi = c.pic_map(x, off, lst)
    ip_w = c.dvc_weights(off, ip_xi)
    c.set_bcs(torch.tensor(mask, device="cuda"))
    c.assemble(off, lst, ip_xi, ip_w, torch.tensor(eta, device="cuda"), torch.tensor(body, device="cuda"))
    opts = dict(rtol=1e-8, inner_rtol=1e-11, outer_rtol=1e-10)
    u0, p0 = c.zeros(m.n_nodes * 2), c.zeros(m.n_el)
    st0 = c.solve(u0, p0, **opts)
    u1, p1 = u0.clone(), p0.clone()
    st1 = c.solve(u1, p1, zero_guess=0, **opts)
    assert st1["pressure_its"] == 0 and st1["residual"] <= 1e-8
    rng = np.random.default_rng(2)
    u2 = u0 + 1e-3 * torch.tensor(rng.standard_normal(u0.shape[0]), device="cuda") * u0.abs().max()
    p2 = p0 + 1e-3 * torch.tensor(rng.standard_normal(p0.shape[0]), device="cuda") * p0.abs().max()
    st2 = c.solve(u2, p2, zero_guess=0, **opts)
    assert st2["residual"] <= 1e-8 and 0 < st2["pressure_its"] < st0["pressure_its"]
    dp = (p2 - p2.mean()) - (p0 - p0.mean())
    assert float((u2 - u0).abs().max()) <= 1e-6 * float(u0.abs().max())
    assert float(dp.abs().max()) <= 1e-6 * float(p0.abs().max())


@pytest.mark.parametrize("res", [(64, 48, 40), (22, 18, 14)])
def test_K32_tiled_apply_many_tiles(gpu, res):
    """The FP32 3D apply (one CTA per 8x8x4 tile; 16-byte weight copies when
    res_x % 4 == 0, else 4-byte) against the FP64 apply: 480 tiles (more than
    the resident CTAs) and a mesh of partial tiles, with
    free-slip walls and scattered interior Dirichlet dofs (tiles with and
    without a Dirichlet flag)."""
    from underworld2_gb300._core import Context, rng_seed
    c = Context(3, res, (0.0,) * 3, (1.0,) * 3)
    x, owner, off, lst, _ = c.layout_random(2, rng_seed(3))
    ip_xi = c.pic_map(x, off, lst)
    ip_w = c.dvc_weights(off, ip_xi, res=6)
    xo = x.cpu().numpy()
    eta = torch.tensor(np.exp(3.0 * np.sin(7.0 * xo[:, 0]) * np.cos(5.0 * xo[:, 2])), device="cuda")
    nodes = np.stack(np.meshgrid(*[np.array(a) for a in reversed(c.axes)], indexing="ij")[::-1], -1).reshape(-1, 3)
    mask = np.zeros((len(nodes), 3), np.uint8)
    for d in range(3):
        mask[:, d] = np.isclose(nodes[:, d], 0.0) | np.isclose(nodes[:, d], 1.0)
    rng = np.random.default_rng(1)
    mask.ravel()[rng.choice(mask.size, 40, replace=False)] = 1
    c.set_bcs(torch.tensor(mask.ravel(), device="cuda"))
    c.assemble(off, lst, ip_xi, ip_w, eta, torch.zeros((len(xo), 3), dtype=torch.float64, device="cuda"))
    xv = rng.standard_normal(mask.size)
    y64 = c.apply_K(torch.tensor(xv, device="cuda")).cpu().numpy()
    y32 = c.apply_K(torch.tensor(xv, device="cuda", dtype=torch.float32)).cpu().numpy()
    assert np.abs(y32 - y64).max() <= 2e-5 * np.abs(y64).max()
    fixed = mask.ravel() != 0
    np.testing.assert_array_equal(y64[fixed], xv[fixed])


@pytest.mark.parametrize("res", [(24, 16, 12), (22, 18, 14)])
def test_K_refine_double_float_matches_fp64(gpu, res):
    """The refinement-residual apply of 3D Q1 (element arithmetic in double-float
    on the FP32 pipe) against the FP64 apply: viscosity contrast e^6, free-slip
    walls plus scattered interior Dirichlet dofs, full and partial tiles.
    Double-float carries about 48 bits: agreement to 1e-12 of max|y|, Dirichlet
    rows equal to x exactly."""
    from underworld2_gb300._core import Context, rng_seed
    c = Context(3, res, (0.0,) * 3, (1.0,) * 3)
    x, owner, off, lst, _ = c.layout_random(4, rng_seed(5))
    ip_xi = c.pic_map(x, off, lst)
    ip_w = c.dvc_weights(off, ip_xi, res=6)
    xo = x.cpu().numpy()
    eta = torch.tensor(np.exp(3.0 * np.sin(5.0 * xo[:, 0]) * np.cos(4.0 * xo[:, 1])), device="cuda")
    nodes = np.stack(np.meshgrid(*[np.array(a) for a in reversed(c.axes)], indexing="ij")[::-1], -1).reshape(-1, 3)
    mask = np.zeros((len(nodes), 3), np.uint8)
    for d in range(3):
        mask[:, d] = np.isclose(nodes[:, d], 0.0) | np.isclose(nodes[:, d], 1.0)
    rng = np.random.default_rng(4)
    mask.ravel()[rng.choice(mask.size, 30, replace=False)] = 1
    c.set_bcs(torch.tensor(mask.ravel(), device="cuda"))
    c.assemble(off, lst, ip_xi, ip_w, eta, torch.zeros((len(xo), 3), dtype=torch.float64, device="cuda"))
    xv = torch.tensor(rng.standard_normal(mask.size), device="cuda")
    y64 = c.apply_K(xv).cpu().numpy()
    ydf = c.apply_K_refine(xv).cpu().numpy()
    assert np.abs(ydf - y64).max() <= 1e-12 * np.abs(y64).max()
    fixed = mask.ravel() != 0
    np.testing.assert_array_equal(ydf[fixed], xv.cpu().numpy()[fixed])


@pytest.mark.parametrize("dim,res,ppc", [(2, (16, 16), 20), (3, (6, 5, 4), 8)])
def test_rk2_fp32_storage_ten_steps(gpu, dim, res, ppc):
    """FP32 particle storage with FP64 arithmetic: ten successive RK2 steps with
    owner updates (migration between elements).  Each GPU step equals the
    oracle's FP64 step from the same stored (widened) coordinates, rounded once
    to FP32; owners and cell tables equal the oracle's after every step."""
    c, m, (x, owner, off, lst), xo, eta, body, mask = _circle_problem(dim, res, ppc)
    ip_xi = c.pic_map(x, off, lst)
    ip_w = c.dvc_weights(off, ip_xi)
    c.set_bcs(torch.tensor(mask, device="cuda"))
    c.assemble(off, lst, ip_xi, ip_w, torch.tensor(eta, device="cuda"), torch.tensor(body, device="cuda"))
    u = c.zeros(m.n_nodes * dim)
    p = c.zeros(m.n_el)
    c.solve(u, p, rtol=1e-8)
    ug = u.cpu().numpy()
    x32 = x.to(torch.float32)
    xo32 = xo.astype(np.float32)
    np.testing.assert_array_equal(x32.cpu().numpy(), xo32)
    tbl, cnt, own_o = m.initial_tables(ppc, 64)
    dt = 3.0 * c.max_dt(u)   # several elements over the ten steps
    for _ in range(10):
        c.rk2(x32, u, dt)
        xn, _ = m.rk2(ug, dt, xo32.astype(np.float64))
        xo32 = xn.astype(np.float32)
        np.testing.assert_array_equal(x32.cpu().numpy(), xo32)
        c.update_owners(x32, owner, off, lst)
        m.update_owners(xo32.astype(np.float64), own_o, tbl, cnt)
        np.testing.assert_array_equal(owner.cpu().numpy(), own_o)
    moved = np.sum(own_o != m.cell_of(xo.astype(np.float32).astype(np.float64)))
    assert moved > 0
    o = off.cpu().numpy()
    lst_h = lst.cpu().numpy()
    for e in range(m.n_el):
        np.testing.assert_array_equal(lst_h[o[e]:o[e + 1]], tbl[e, : cnt[e]])
