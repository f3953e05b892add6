"""GPU parity of the 3D Q2/dPc1 path against the CPU oracle (through the C ABI).

Bit-exact: particle layout, ownership, local coordinates (Newton with the
reference's triquadratic basis), DVC weights and RK2 positions.  Tolerances:
element matrices 1e-10 relative (FP64), operator applies 1e-12 (FP64) and 1e-5
(FP32), solutions 1e-7 of the field scale with both sides converged.  The
pressure is dPc1 with four coefficients per element
(TrilinearInnerElType.c:202-215); the Schur preconditioner is the reference's
Uzawa term, a 4x4 block per element.
"""
import numpy as np
import pytest
import torch

import oracle
from tests import oracle_system

pytestmark = pytest.mark.gpu


def _problem(res, ppc, seed=21):
    from underworld2_gb300._core import Context, rng_seed
    c = Context(3, res, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), order=2, porder=1)
    m = oracle.Mesh(3, 2, res, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), porder=1)
    x, owner, off, lst, _ = c.layout_random(ppc, rng_seed(seed))
    xo, _ = m.layout_random(ppc, seed)
    dense = xo[:, 2] > 0.3 + 0.05 * np.cos(np.pi * xo[:, 0]) * np.cos(np.pi * xo[:, 1])
    rng = np.random.default_rng(seed)
    eta = np.where(dense, 1.0, 0.05) * 10.0 ** rng.uniform(-0.5, 0.5, len(xo))
    body = np.zeros((len(xo), 3))
    body[:, 2] = np.where(dense, -1.0, 0.0)
    nodes = m.node_coords()
    mask = np.zeros((m.n_nodes, 3), np.uint8)
    for d in range(3):
        mask[:, d] = (np.isclose(nodes[:, d], 0.0) | np.isclose(nodes[:, d], 1.0)).astype(np.uint8)
    return c, m, (x, owner, off, lst), xo, eta, body, mask.ravel()


def _assembled(res, ppc):
    c, m, (x, owner, off, lst), xo, eta, body, mask = _problem(res, ppc)
    ip_xi = c.pic_map(x, off, lst)
    ip_w = c.dvc_weights(off, ip_xi)
    c.set_bcs(torch.tensor(mask, device="cuda"))
    c.assemble(off, lst, ip_xi, ip_w, torch.tensor(eta, device="cuda"), torch.tensor(body, device="cuda"))
    tbl, cnt, _ = m.initial_tables(ppc, ppc)
    oxi, ow = m.pic_map(xo, tbl, cnt)
    pts = oracle_system.pic_points_by_element(tbl, cnt, oxi, ow)
    return c, m, (x, owner, off, lst), xo, eta, body, mask, (tbl, cnt, oxi, ow), pts


def test_q2_3d_particles_bit_exact(gpu):
    res, ppc = (3, 3, 2), 12
    c, m, (x, owner, off, lst), xo, eta, body, mask = _problem(res, ppc)
    np.testing.assert_array_equal(x.cpu().numpy(), xo)
    np.testing.assert_array_equal(c.locate(x).cpu().numpy(), m.cell_of(xo))
    ip_xi = c.pic_map(x, off, lst)
    tbl, cnt, _ = m.initial_tables(ppc, ppc)
    slots = np.concatenate([tbl[e, : cnt[e]] for e in range(m.n_el)])
    gxi = np.array([m.global_to_local(m.cell_of(xo[p : p + 1])[0], xo[p])[0] for p in slots])
    np.testing.assert_array_equal(ip_xi.cpu().numpy(), gxi)
    ip_w = c.dvc_weights(off, ip_xi)
    oxi, ow = m.pic_map(xo, tbl, cnt)
    np.testing.assert_array_equal(ip_xi.cpu().numpy(), oxi[slots])
    np.testing.assert_array_equal(ip_w.cpu().numpy(), ow[slots])


def test_q2_3d_element_matrices_and_operators(gpu):
    c, m, _, xo, eta, body, mask, _, pts = _assembled((3, 2, 2), 16)
    gxi, gw = m.gauss_points()
    for e in [0, 5, m.n_el - 1]:
        Ke, Ge, Se = c.element_matrices(e)
        ps, xi, w = pts[e]
        Ko = m.element_K(e, xi, w, eta[ps])
        assert np.abs(Ke - Ko).max() <= 1e-10 * np.abs(Ko).max()
        Go = m.element_G(e, gxi, gw)
        assert np.abs(Ge - Go).max() <= 1e-12 * np.abs(Go).max()
        So = m.element_S(Ko, Go)
        assert np.abs(Se - So).max() <= 1e-10 * np.abs(So).max()
    sysd = oracle_system.assemble(m, pts, eta, body, mask, np.zeros(len(mask)))
    rng = np.random.default_rng(1)
    free = mask == 0
    xv = rng.standard_normal(m.n_nodes * 3) * free
    y = c.apply_K(torch.tensor(xv, device="cuda")).cpu().numpy()
    yo = sysd["K"] @ xv
    assert np.abs(y[free] - yo[free]).max() <= 1e-12 * np.abs(yo).max()
    y32 = c.apply_K(torch.tensor(xv, device="cuda", dtype=torch.float32)).cpu().numpy()
    assert np.abs(y32[free] - yo[free]).max() <= 1e-5 * np.abs(yo).max()
    # refinement residuals: double-float element matrices, about 2^-48 relative
    yr = c.apply_K_refine(torch.tensor(xv, device="cuda")).cpu().numpy()
    assert np.abs(yr[free] - yo[free]).max() <= 1e-12 * np.abs(yo).max()
    np.testing.assert_array_equal(yr[~free], xv[~free])
    pv = rng.standard_normal(m.n_el * 4)
    yg = c.apply_G(torch.tensor(pv, device="cuda")).cpu().numpy()
    assert np.abs(yg[free] - (sysd["G"] @ pv)[free]).max() <= 1e-12 * np.abs(yg).max()
    q = c.apply_Gt(torch.tensor(xv, device="cuda")).cpu().numpy()
    assert np.abs(q - sysd["G"].T @ xv).max() <= 1e-12 * np.abs(q).max()


@pytest.mark.parametrize("mixed", [0, 1])
def test_q2_3d_solve_matches_direct_and_advects(gpu, mixed):
    res, ppc = (3, 3, 3), 12
    c, m, (x, owner, off, lst), xo, eta, body, mask, (tbl, cnt, oxi, ow), pts = _assembled(res, ppc)
    u = c.zeros(m.n_nodes * 3)
    p = c.zeros(m.n_el * 4)
    st = c.solve(u, p, mixed=mixed, schur_pc=0, rtol=1e-8, inner_rtol=1e-11, outer_rtol=1e-10)
    assert st["residual"] <= 1e-8, st
    sysd = oracle_system.assemble(m, pts, eta, body, mask, np.zeros(len(mask)))
    uo, po = oracle_system.solve(sysd, m.n_nodes * 3)
    ug, pg = u.cpu().numpy(), p.cpu().numpy()
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
