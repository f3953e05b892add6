"""Coarse-level correction of the Schur-complement flexible GMRES (GPU).

The deflation step z = y + Q (r - S y) with the Galerkin coarse Schur
complement (uwg_coarse.cu) on the learned part's random 2D problems (log10
viscosity Gaussian random field with contrast 1e3-1e6 plus buoyant
inclusions, 128^2 Q1/dQ0, free slip): every solve reaches the same 1e-8
residual and the same solution as the plain solve, with fewer outer
iterations in total.  Plus the argument checks and the cases the correction
does not apply to (compressible block, checkerboard null space).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_fewer_outer_iterations_same_solution(gpu):
    from underworld2_gb300 import learned
    ps = learned.ProblemSet(res=128, ppc=12)
    plain_its = coarse_its = 0
    for seed in (101, 102, 103, 104):
        ps.assemble(seed)
        u0, p0, st0 = ps.solve(1)
        ctx = ps.ctx
        u1, p1 = ctx.zeros(ctx.n_vdof), ctx.zeros(ctx.n_pdof)
        st1 = ctx.solve(u1, p1, mixed=1, rtol=1e-8, inner_rtol=1e-10, outer_rtol=1e-9, smooth_steps=2, restart=120,
                        schur_pc=1, max_outer=500, coarse_agg=8)
        assert st1["coarse_dim"] == 256 and st1["residual"] <= 1e-8 and st0["residual"] <= 1e-8
        du = float((u1 - u0).norm() / u0.norm())
        dp = float(((p1 - p1.mean()) - (p0 - p0.mean())).norm() / (p0 - p0.mean()).norm())
        assert du <= 1e-6 and dp <= 1e-6, (seed, du, dp)
        plain_its += st0["pressure_its"]
        coarse_its += st1["pressure_its"]
    assert coarse_its < 0.75 * plain_its, (coarse_its, plain_its)


def test_arguments_and_inapplicable_cases(gpu):
    from underworld2_gb300 import _native
    from underworld2_gb300._core import Context, rng_seed
    c = Context(2, (32, 32), (0.0, 0.0), (1.0, 1.0))
    n = 33
    idx = np.arange(n * n)
    mask = np.zeros((n * n, 2), np.uint8)
    mask[:, 0] = (idx % n == 0) | (idx % n == n - 1)
    mask[:, 1] = (idx // n == 0) | (idx // n == n - 1)
    c.set_bcs(torch.tensor(mask.ravel(), device="cuda"))
    x, owner, off, lst, _ = c.layout_random(8, rng_seed(5))
    ip_xi = c.pic_map(x, off, lst)
    ip_w = c.dvc_weights(off, ip_xi)
    eta = torch.ones(x.shape[0], dtype=torch.float64, device="cuda")
    body = torch.zeros_like(x)
    body[:, 1] = -torch.where(((x - 0.5) ** 2).sum(1) < 0.04, 1.0, 0.0)
    c.assemble(off, lst, ip_xi, ip_w, eta, body)
    u, p = c.zeros(c.n_vdof), c.zeros(c.n_pdof)
    for bad in (3, 6, 64):     # odd; does not divide 32; no velocity level 1 element wide on a 1 x 1 grid
        with pytest.raises(_native.UwgError):
            c.solve(u, p, coarse_agg=bad)
    st = c.solve(u, p, coarse_agg=4)
    assert st["coarse_dim"] == 64 and st["residual"] <= 1e-8
    # compressible block: BFBt is replaced by the Uzawa term and the correction is not applied
    c.assemble(off, lst, ip_xi, ip_w, eta, body, torch.full_like(eta, 1e-3))
    st = c.solve(c.zeros(c.n_vdof), c.zeros(c.n_pdof), coarse_agg=4)
    assert st["coarse_dim"] == 0 and st["schur_pc_used"] == 0
    # every wall fixed (checkerboard null mode): not applied
    c.set_bcs(torch.ones(2 * n * n, dtype=torch.uint8, device="cuda"))
    c.assemble(off, lst, ip_xi, ip_w, eta, body)
    st = c.solve(c.zeros(c.n_vdof), c.zeros(c.n_pdof), coarse_agg=4, null_space=2)
    assert st["coarse_dim"] == 0
