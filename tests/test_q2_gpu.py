"""GPU parity of the 2D Q2/dPc1 path against the CPU oracle (through the C ABI).

Bit-exact: particle layout, ownership, local coordinates, DVC weights and RK2
positions on the biquadratic mesh.  Tolerance: element matrices 1e-10
relative (FP64), operator applies 1e-12, solutions 1e-7 of the field scale
with both sides converged.  The pressure is dPc1 (three coefficients per
element; BilinearInnerElType.c:169-179) and the Schur preconditioner is the
reference's Uzawa term, a 3x3 block per element.
"""
import numpy as np
import pytest
import torch

import oracle
from tests import oracle_system

pytestmark = pytest.mark.gpu


def _rt_problem(res, ppc, seed=13):
    """Rayleigh-Taylor layering: dense (rho 1, eta 1) above y = 0.2 + 0.02 cos(pi x),
    light (rho 0, eta 0.01) below, per-particle eta times 10^U(-1, 1); free slip."""
    from underworld2_gb300._core import Context, rng_seed
    c = Context(2, res, (0.0, 0.0), (1.0, 1.0), order=2, porder=1)
    m = oracle.Mesh(2, 2, res, (0.0, 0.0), (1.0, 1.0), porder=1)
    x, owner, off, lst, _ = c.layout_random(ppc, rng_seed(seed))
    xo, _ = m.layout_random(ppc, seed)
    dense = xo[:, 1] > 0.2 + 0.02 * np.cos(np.pi * xo[:, 0])
    rng = np.random.default_rng(seed)
    eta = np.where(dense, 1.0, 0.01) * 10.0 ** rng.uniform(-1.0, 1.0, len(xo))
    body = np.zeros((len(xo), 2))
    body[:, 1] = np.where(dense, -1.0, 0.0)
    nodes = m.node_coords()
    mask = np.zeros((m.n_nodes, 2), np.uint8)
    for d in range(2):
        mask[:, d] = (np.isclose(nodes[:, d], 0.0) | np.isclose(nodes[:, d], 1.0)).astype(np.uint8)
    return c, m, (x, owner, off, lst), xo, eta, body, mask.ravel()


def _assembled(res, ppc):
    c, m, (x, owner, off, lst), xo, eta, body, mask = _rt_problem(res, ppc)
    ip_xi = c.pic_map(x, off, lst)
    ip_w = c.dvc_weights(off, ip_xi)
    c.set_bcs(torch.tensor(mask, device="cuda"))
    c.assemble(off, lst, ip_xi, ip_w, torch.tensor(eta, device="cuda"), torch.tensor(body, device="cuda"))
    tbl, cnt, _ = m.initial_tables(ppc, ppc)
    oxi, ow = m.pic_map(xo, tbl, cnt)
    pts = oracle_system.pic_points_by_element(tbl, cnt, oxi, ow)
    return c, m, (x, owner, off, lst), xo, eta, body, mask, (ip_xi, ip_w), (tbl, cnt, oxi, ow), pts


@pytest.mark.parametrize("res,ppc", [((6, 5), 12), ((4, 4), 20)])
def test_q2_particles_bit_exact(gpu, res, ppc):
    c, m, (x, owner, off, lst), xo, eta, body, mask = _rt_problem(res, ppc)
    np.testing.assert_array_equal(x.cpu().numpy(), xo)
    np.testing.assert_array_equal(c.locate(x).cpu().numpy(), m.cell_of(xo))
    ip_xi = c.pic_map(x, off, lst)
    ip_w = c.dvc_weights(off, ip_xi)
    tbl, cnt, _ = m.initial_tables(ppc, ppc)
    oxi, ow = m.pic_map(xo, tbl, cnt)
    slots = np.concatenate([tbl[e, : cnt[e]] for e in range(m.n_el)])
    np.testing.assert_array_equal(ip_xi.cpu().numpy(), oxi[slots])
    np.testing.assert_array_equal(ip_w.cpu().numpy(), ow[slots])


def test_q2_element_matrices_and_operators(gpu):
    c, m, _, xo, eta, body, mask, _, _, pts = _assembled((6, 5), 20)
    gxi, gw = m.gauss_points()
    for e in [0, 7, m.n_el - 1]:
        Ke, Ge, Se = c.element_matrices(e)
        ps, xi, w = pts[e]
        Ko = m.element_K(e, xi, w, eta[ps])
        assert np.abs(Ke - Ko).max() <= 1e-10 * np.abs(Ko).max()
        Go = m.element_G(e, gxi, gw)
        assert np.abs(Ge - Go).max() <= 1e-12 * np.abs(Go).max()
        So = m.element_S(Ko, Go)
        assert np.abs(Se - So).max() <= 1e-10 * np.abs(So).max()
    sysd = oracle_system.assemble(m, pts, eta, body, mask, np.zeros(len(mask)))
    rng = np.random.default_rng(0)
    free = mask == 0
    xv = rng.standard_normal(m.n_nodes * 2) * free
    y = c.apply_K(torch.tensor(xv, device="cuda")).cpu().numpy()
    yo = sysd["K"] @ xv
    assert np.abs(y[free] - yo[free]).max() <= 1e-12 * np.abs(yo).max()
    y32 = c.apply_K(torch.tensor(xv, device="cuda", dtype=torch.float32)).cpu().numpy()
    assert np.abs(y32[free] - yo[free]).max() <= 1e-5 * np.abs(yo).max()
    pv = rng.standard_normal(m.n_el * 3)
    yg = c.apply_G(torch.tensor(pv, device="cuda")).cpu().numpy()
    assert np.abs(yg[free] - (sysd["G"] @ pv)[free]).max() <= 1e-12 * np.abs(yg).max()
    q = c.apply_Gt(torch.tensor(xv, device="cuda")).cpu().numpy()
    assert np.abs(q - sysd["G"].T @ xv).max() <= 1e-12 * np.abs(q).max()


@pytest.mark.parametrize("mixed", [0, 1])
def test_q2_solve_matches_direct_and_advects(gpu, mixed):
    res, ppc = (8, 8), 20
    c, m, (x, owner, off, lst), xo, eta, body, mask, _, (tbl, cnt, oxi, ow), pts = _assembled(res, ppc)
    u = c.zeros(m.n_nodes * 2)
    p = c.zeros(m.n_el * 3)
    st = c.solve(u, p, mixed=mixed, schur_pc=0, rtol=1e-8, inner_rtol=1e-11, outer_rtol=1e-10)
    assert st["residual"] <= 1e-8, st
    sysd = oracle_system.assemble(m, pts, eta, body, mask, np.zeros(len(mask)))
    uo, po = oracle_system.solve(sysd, m.n_nodes * 2)
    ug, pg = u.cpu().numpy(), p.cpu().numpy()
    # the constant pressure (all dPc1 coefficients equal) is the null space under free slip
    pg = pg - pg.mean()
    po = po - po.mean()
    assert np.abs(ug - uo).max() <= 1e-7 * np.abs(uo).max()
    assert np.abs(pg - po).max() <= 1e-7 * np.abs(po).max()
    dt = c.max_dt(u)
    x_gpu = x.clone()
    fb, failed = c.rk2(x_gpu, u, dt)
    x_or, counts = m.rk2(ug, dt, xo.copy())
    assert failed == counts[0] and fb == counts[1]
    np.testing.assert_array_equal(x_gpu.cpu().numpy(), x_or)


def test_q2_rejects_bfbt(gpu):
    from underworld2_gb300 import _native
    c, m, *_ = _assembled((4, 4), 12)
    u = c.zeros(m.n_nodes * 2)
    p = c.zeros(m.n_el * 3)
    with pytest.raises(_native.UwgError):
        c.solve(u, p, schur_pc=1)
