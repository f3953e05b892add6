"""The learned warm start's kernels and its use in the solve (GPU).

BF16 tensor-core GEMM (all operand layouts, bias, ReLU, accumulation, BF16
output) against torch FP32 on the same BF16 inputs; convolution forward and
backward against torch autograd; pooling and upsampling against torch; a few
Adam steps reduce the loss; a warm-started solve reaches the same FP64
residual and solution as the plain solve, and a network that returns garbage
falls back to the plain FP64 solve.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ctx():
    from underworld2_gb300._core import Context
    return Context(2, (8, 8), (0.0, 0.0), (1.0, 1.0))


@pytest.mark.parametrize("at,bt", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_gemm_matches_torch(gpu, at, bt):
    from underworld2_gb300.learned import _Ops
    ops = _Ops(_ctx())
    g = torch.Generator(device="cuda").manual_seed(at * 2 + bt)
    M, N, K = 150, 70, 93
    A = torch.randn((K, M) if at else (M, K), device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn((N, K) if bt else (K, N), device="cuda", generator=g).to(torch.bfloat16)
    bias = torch.randn(N, device="cuda", generator=g)
    Af = A.float().t() if at else A.float()
    Bf = B.float().t() if bt else B.float()
    ref = Af @ Bf + bias
    C = torch.empty((M, N), device="cuda")
    Cb = torch.empty((M, N), device="cuda", dtype=torch.bfloat16)
    ops.gemm(M, N, K, A, M if at else K, at, B, K if bt else N, bt, Cf=C, Cb=Cb, ldc=N, bias=bias)
    torch.cuda.synchronize()
    assert torch.allclose(C, ref, rtol=1e-4, atol=1e-3 * ref.abs().max().item())
    assert torch.allclose(Cb.float(), ref, rtol=1e-2, atol=1e-2 * ref.abs().max().item())
    C2 = C.clone()
    ops.gemm(M, N, K, A, M if at else K, at, B, K if bt else N, bt, Cf=C2, ldc=N, relu=True, acc=True)
    assert torch.allclose(C2, torch.relu(C + Af @ Bf), rtol=1e-4, atol=1e-3 * ref.abs().max().item())


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (300, 32, 72), (1000, 96, 288), (257, 128, 576),
                                   (4096, 256, 1152), (77, 200, 1000), (130, 3, 288)])
def test_tcgen05_gemm_matches_torch_fp32(gpu, M, N, K):
    """The tcgen05 GEMM (K-major A and B, accumulator in tensor memory) against torch's
    FP32 matmul and the mma.sync kernel on the same BF16 inputs: ragged M and N, K
    not a multiple of the 64-wide chunk, bias, ReLU, accumulation and a BF16 copy."""
    from underworld2_gb300.learned import _Ops
    ops = _Ops(_ctx())
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn((M, K), device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn((N, K), device="cuda", generator=g).to(torch.bfloat16)
    bias = torch.randn(N, device="cuda", generator=g)
    ref = A.float() @ B.float().t() + bias
    bound = 1e-5 * (A.float().abs() @ B.float().abs().t()).max().item()
    C = torch.full((M, N), float("nan"), device="cuda")
    Cb = torch.empty((M, N), device="cuda", dtype=torch.bfloat16)
    ops.gemm(M, N, K, A, K, 0, B, K, 1, Cf=C, Cb=Cb, ldc=N, bias=bias)
    ops.check()
    assert (C - ref).abs().max().item() <= bound
    assert torch.equal(Cb, C.to(torch.bfloat16))
    ops.set_path(1)
    C1 = torch.empty((M, N), device="cuda")
    ops.gemm(M, N, K, A, K, 0, B, K, 1, Cf=C1, ldc=N, bias=bias)
    ops.set_path(0)
    assert (C - C1).abs().max().item() <= bound
    C2 = C.clone()
    ops.gemm(M, N, K, A, K, 0, B, K, 1, Cf=C2, ldc=N, relu=True, acc=True)
    ops.check()
    assert (C2 - torch.relu(C + A.float() @ B.float().t())).abs().max().item() <= 2 * bound


def test_conv_forward_backward_matches_autograd(gpu):
    from underworld2_gb300.learned import Conv3x3, _Ops
    ops = _Ops(_ctx())
    gen = torch.Generator().manual_seed(3)
    conv = Conv3x3(5, 12, True, gen, "cuda")
    conv.b.copy_(torch.randn(12, generator=gen).cuda() * 0.1)
    x = torch.randn((2, 10, 12, 5), device="cuda").to(torch.bfloat16)
    y = conv.forward(ops, x, out_float=True)
    xt = x.float().permute(0, 3, 1, 2).clone().requires_grad_(True)
    wt = conv.wb.float().reshape(12, 3, 3, 5).permute(0, 3, 1, 2).clone().requires_grad_(True)
    bt = conv.b.clone().requires_grad_(True)
    ref = torch.relu(torch.nn.functional.conv2d(xt, wt, bt, padding=1))
    assert torch.allclose(y.permute(0, 3, 1, 2), ref, rtol=1e-3, atol=1e-3)
    gy = torch.randn_like(ref)
    ref.backward(gy)
    ybf = y.to(torch.bfloat16)
    gx = conv.backward(ops, x, ybf, gy.permute(0, 2, 3, 1).contiguous().clone())
    torch.cuda.synchronize()
    gw = conv.gw.reshape(12, 3, 3, 5).permute(0, 3, 1, 2)
    scale = lambda t: t.abs().max().item()
    assert (gw - wt.grad).abs().max().item() <= 2e-2 * scale(wt.grad)
    assert (conv.gb - bt.grad).abs().max().item() <= 2e-2 * scale(bt.grad)
    assert (gx.permute(0, 3, 1, 2) - xt.grad).abs().max().item() <= 2e-2 * scale(xt.grad)


def test_pool_and_upsample(gpu):
    from underworld2_gb300.learned import WarmStartNet
    net = WarmStartNet(_ctx(), base=8)
    x = torch.randn((2, 8, 6, 3), device="cuda").to(torch.bfloat16)
    p = net._pool(x)
    ref = torch.nn.functional.avg_pool2d(x.float().permute(0, 3, 1, 2), 2).permute(0, 2, 3, 1)
    assert torch.allclose(p.float(), ref, rtol=1e-2, atol=1e-2)
    u = net._up(p)
    assert torch.equal(u.float(), p.float().repeat_interleave(2, 1).repeat_interleave(2, 2))
    g = torch.randn((2, 8, 6, 3), device="cuda")
    gp = net._up_bwd(g)
    assert torch.allclose(gp, torch.nn.functional.avg_pool2d(g.permute(0, 3, 1, 2), 2).permute(0, 2, 3, 1) * 4,
                          rtol=1e-5, atol=1e-5)


def test_training_reduces_loss(gpu):
    from underworld2_gb300.learned import WarmStartNet
    net = WarmStartNet(_ctx(), seed=1, base=8)
    g = torch.Generator(device="cuda").manual_seed(0)
    X = torch.randn((4, 16, 16, 3), device="cuda", generator=g)
    Y = torch.stack([X[..., 0], X[..., 1], X[..., 2] - X[..., 1]], -1)
    l0 = net.train_step(X.to(torch.bfloat16), Y, 3e-3)
    for _ in range(150):
        l1 = net.train_step(X.to(torch.bfloat16), Y, 3e-3)
    assert np.isfinite(l1) and l1 < 0.4 * l0


def test_warm_start_solve_and_fallback(gpu):
    from underworld2_gb300 import learned
    ps = learned.ProblemSet(res=32, ppc=12)
    net = learned.WarmStartNet(ps.ctx, seed=2, base=8)
    f, scales = ps.assemble(11)
    u0, p0, st0 = ps.solve(0)
    u1, p1, st1, fb = learned.solve_with_warm_start(ps, net, f, scales)
    assert not fb and st1["residual"] <= 1e-8 and st0["residual"] <= 1e-8
    du = (u1 - u0).abs().max().item() / u0.abs().max().item()
    pm = lambda p: p - p.mean()
    dp = (pm(p1) - pm(p0)).abs().max().item() / pm(p0).abs().max().item()
    assert du < 1e-6 and dp < 1e-6
    u3, p3, st3, fb3 = learned.solve_with_warm_start(ps, net, f, scales, mode="guess")
    assert not fb3 and st3["residual"] <= 1e-8
    # the exact pressure as the first search direction: one Schur iteration suffices
    u4, p4, st4 = ps.solve(1, p_dir=p0 - p0.mean())
    assert st4["residual"] <= 1e-8 and st4["pressure_its"] <= 2 < st0["pressure_its"]
    # a network returning garbage: the plain FP64 solve takes over
    net.out.b.fill_(float("nan"))
    u2, p2, st2, fb2 = learned.solve_with_warm_start(ps, net, f, scales)
    assert fb2 and st2["residual"] <= 1e-8
