"""Learned warm start for the Stokes solve.

A small convolutional network (about 1.16M parameters, 4 resolution levels,
32 base channels, encoder-decoder with additive skips) maps per-cell
log10-viscosity and buoyancy of a 2D Q1/dQ0 problem (with the buoyancy's
column integral, the hydrostatic pressure, as a third input) to the cell
velocity and pressure.  It is trained on solves of this library's own BSSCR path, and its
pressure is the initial guess of the Schur FGMRES (``zero_guess = 0``); the
velocity channels are trained alongside but the BSSCR iteration only takes a
pressure guess.  Every convolution runs as BF16 tensor-core GEMMs with FP32
accumulation in libuwg (``uwg_cnn_*``, hand-written forward and backward; the
forward product on tcgen05 with the accumulator in tensor memory); the
master weights, gradients and Adam moments are FP32.  PyTorch holds the device
buffers and does the few gradient additions of the skip connections.

The plain path decides every result: a warm-started solve reports the same FP64
residual as any other, and ``solve_with_warm_start`` falls back to the plain
FP64 solve when the warm-started mixed-precision solve does not reach the
tolerance.
"""
import ctypes
import math

import numpy as np
import torch

from . import _native

_BF = torch.bfloat16


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class _Ops:
    """Thin wrappers of the uwg_cnn_* entry points on one context's stream."""

    def __init__(self, ctx):
        self.ctx = ctx

    def gemm(self, M, N, K, A, lda, at, B, ldb, bt, Cf=None, Cb=None, ldc=None, bias=None, relu=False, acc=False):
        self.ctx._call("uwg_cnn_gemm", int(M), int(N), int(K), _p(A), int(lda), int(at), _p(B), int(ldb), int(bt),
                       _p(Cf), _p(Cb), int(ldc), _p(bias), int(relu), int(acc))

    def check(self):
        """Synchronise; raises if a tensor-core GEMM gave up a bounded wait."""
        self.ctx._call("uwg_cnn_check")

    def set_path(self, path):
        """0: tcgen05 GEMM where the operands allow it (default); 1: mma.sync always."""
        self.ctx._call("uwg_cnn_set_path", int(path))

    def im2col(self, nb, H, W, C, x, col):
        self.ctx._call("uwg_cnn_im2col", nb, H, W, C, _p(x), _p(col))

    def col2im(self, nb, H, W, C, col, out):
        self.ctx._call("uwg_cnn_col2im", nb, H, W, C, _p(col), _p(out))

    def ew(self, op, nb, H, W, C, a16=None, b16=None, c16=None, fa=None, fb=None):
        self.ctx._call("uwg_cnn_elementwise", op, nb, H, W, C, _p(a16), _p(b16), _p(c16), _p(fa), _p(fb))


class Conv3x3:
    """3x3 convolution (zero padding) with bias and optional ReLU on NHWC tensors."""

    def __init__(self, cin, cout, relu, gen, device):
        self.cin, self.cout, self.relu = cin, cout, relu
        std = math.sqrt(2.0 / (9 * cin)) if relu else math.sqrt(1.0 / (9 * cin))
        self.w = (torch.randn(cout, 9 * cin, generator=gen, dtype=torch.float32) * std).to(device)
        self.b = torch.zeros(cout, dtype=torch.float32, device=device)
        self.wb = self.w.to(_BF)
        self.gw, self.gb = torch.zeros_like(self.w), torch.zeros_like(self.b)
        self.state = [torch.zeros_like(self.w), torch.zeros_like(self.w), torch.zeros_like(self.b),
                      torch.zeros_like(self.b)]

    def n_params(self):
        return self.w.numel() + self.b.numel()

    def forward(self, ops, x, out_float=False):
        nb, H, W, C = x.shape
        P = nb * H * W
        col = torch.empty((P, 9 * C), dtype=_BF, device=x.device)
        ops.im2col(nb, H, W, C, x, col)
        if out_float:
            y = torch.empty((nb, H, W, self.cout), dtype=torch.float32, device=x.device)
            ops.gemm(P, self.cout, 9 * C, col, 9 * C, 0, self.wb, 9 * C, 1, Cf=y, ldc=self.cout, bias=self.b,
                     relu=self.relu)
        else:
            y = torch.empty((nb, H, W, self.cout), dtype=_BF, device=x.device)
            ops.gemm(P, self.cout, 9 * C, col, 9 * C, 0, self.wb, 9 * C, 1, Cb=y, ldc=self.cout, bias=self.b,
                     relu=self.relu)
        return y

    def backward(self, ops, x, y, gy, need_gx=True):
        """gy: FP32 gradient of the output (modified in place by the ReLU mask)."""
        nb, H, W, C = x.shape
        P = nb * H * W
        if self.relu:
            ops.ew(0, 1, 1, 1, P * self.cout, a16=y, fb=gy)
        self.ctx_bias(ops, P, gy)
        gy16 = torch.empty((P, self.cout), dtype=_BF, device=x.device)
        ops.ew(6, 1, 1, 1, P * self.cout, fa=gy, c16=gy16)
        col = torch.empty((P, 9 * C), dtype=_BF, device=x.device)
        ops.im2col(nb, H, W, C, x, col)
        ops.gemm(self.cout, 9 * C, P, gy16, self.cout, 1, col, 9 * C, 0, Cf=self.gw, ldc=9 * C)
        if not need_gx:
            return None
        dcol = torch.empty((P, 9 * C), dtype=torch.float32, device=x.device)
        ops.gemm(P, 9 * C, self.cout, gy16, self.cout, 0, self.wb, 9 * C, 0, Cf=dcol, ldc=9 * C)
        gx = torch.empty((nb, H, W, C), dtype=torch.float32, device=x.device)
        ops.col2im(nb, H, W, C, dcol, gx)
        return gx

    def ctx_bias(self, ops, P, gy):
        ops.ctx._call("uwg_cnn_bias_grad", int(P), self.cout, _p(gy), _p(self.gb))

    def adam(self, ops, step, lr, b1=0.9, b2=0.999, eps=1e-8):
        mw, vw, mb, vb = self.state
        ops.ctx._call("uwg_cnn_adam", self.w.numel(), _p(self.w), _p(self.gw), _p(mw), _p(vw), _p(self.wb),
                      ctypes.c_float(lr), ctypes.c_float(b1), ctypes.c_float(b2), ctypes.c_float(eps), step)
        ops.ctx._call("uwg_cnn_adam", self.b.numel(), _p(self.b), _p(self.gb), _p(mb), _p(vb), None,
                      ctypes.c_float(lr), ctypes.c_float(b1), ctypes.c_float(b2), ctypes.c_float(eps), step)


class WarmStartNet:
    """Encoder-decoder CNN: 3 input channels (log10 viscosity / 3, buoyancy,
    scaled hydrostatic pressure) on an
    H x W cell grid (H, W divisible by 8) -> 3 output channels (viscosity-scaled
    velocity x and y, pressure) per cell."""

    def __init__(self, ctx, seed=0, base=32):
        self.ops = _Ops(ctx)
        dev = ctx.device
        g = torch.Generator().manual_seed(seed)
        c1, c2, c3, c4 = base, 2 * base, 4 * base, 8 * base
        C = lambda a, b, r=True: Conv3x3(a, b, r, g, dev)
        self.e1a, self.e1 = C(3, c1), C(c1, c1)
        self.e2a, self.e2 = C(c1, c2), C(c2, c2)
        self.e3a, self.e3 = C(c2, c3), C(c3, c3)
        self.bt = C(c3, c4)
        self.d3a, self.d3 = C(c4, c3), C(c3, c3)
        self.d2a, self.d2 = C(c3, c2), C(c2, c2)
        self.d1a, self.d1 = C(c2, c1), C(c1, c1)
        self.out = C(c1, 3, False)
        self.layers = [self.e1a, self.e1, self.e2a, self.e2, self.e3a, self.e3, self.bt, self.d3a, self.d3,
                       self.d2a, self.d2, self.d1a, self.d1, self.out]
        self.step = 0
        # per-channel scale of the targets (set from the training set by ``train``)
        self.scale = torch.ones(3, dtype=torch.float32, device=dev)

    def n_params(self):
        return sum(l.n_params() for l in self.layers)

    def _pool(self, x):
        nb, H, W, C = x.shape
        y = torch.empty((nb, H // 2, W // 2, C), dtype=_BF, device=x.device)
        self.ops.ew(1, nb, H, W, C, a16=x, c16=y)
        return y

    def _up(self, x):
        nb, H, W, C = x.shape
        y = torch.empty((nb, 2 * H, 2 * W, C), dtype=_BF, device=x.device)
        self.ops.ew(3, nb, H, W, C, a16=x, c16=y)
        return y

    def _add(self, a, b):
        y = torch.empty_like(a)
        self.ops.ew(5, 1, 1, 1, a.numel(), a16=a, b16=b, c16=y)
        return y

    def _pool_bwd(self, g, H, W):
        nb, _, _, C = g.shape
        out = torch.empty((nb, H, W, C), dtype=torch.float32, device=g.device)
        self.ops.ew(2, nb, H, W, C, fa=g, fb=out)
        return out

    def _up_bwd(self, g):
        nb, H2, W2, C = g.shape
        out = torch.empty((nb, H2 // 2, W2 // 2, C), dtype=torch.float32, device=g.device)
        self.ops.ew(4, nb, H2 // 2, W2 // 2, C, fa=g, fb=out)
        return out

    def forward(self, x):
        """x: [nb, H, W, 3] BF16 -> [nb, H, W, 3] FP32; activations kept for backward."""
        o = self.ops
        a = {"x": x}
        a["e1a"] = self.e1a.forward(o, x)
        a["e1"] = self.e1.forward(o, a["e1a"])
        a["p1"] = self._pool(a["e1"])
        a["e2a"] = self.e2a.forward(o, a["p1"])
        a["e2"] = self.e2.forward(o, a["e2a"])
        a["p2"] = self._pool(a["e2"])
        a["e3a"] = self.e3a.forward(o, a["p2"])
        a["e3"] = self.e3.forward(o, a["e3a"])
        a["p3"] = self._pool(a["e3"])
        a["bt"] = self.bt.forward(o, a["p3"])
        a["u3"] = self._up(a["bt"])
        a["d3a"] = self.d3a.forward(o, a["u3"])
        a["s3"] = self._add(a["d3a"], a["e3"])
        a["d3"] = self.d3.forward(o, a["s3"])
        a["u2"] = self._up(a["d3"])
        a["d2a"] = self.d2a.forward(o, a["u2"])
        a["s2"] = self._add(a["d2a"], a["e2"])
        a["d2"] = self.d2.forward(o, a["s2"])
        a["u1"] = self._up(a["d2"])
        a["d1a"] = self.d1a.forward(o, a["u1"])
        a["s1"] = self._add(a["d1a"], a["e1"])
        a["d1"] = self.d1.forward(o, a["s1"])
        a["y"] = self.out.forward(o, a["d1"], out_float=True)
        self._acts = a
        return a["y"]

    def backward(self, gy):
        """gy: FP32 [nb, H, W, 3] gradient of the loss w.r.t. the output."""
        o, a = self.ops, self._acts
        g = self.out.backward(o, a["d1"], a["y"], gy)
        g = self.d1.backward(o, a["s1"], a["d1"], g)
        g_e1 = g.clone()
        g = self.d1a.backward(o, a["u1"], a["d1a"], g)
        g = self._up_bwd(g)
        g = self.d2.backward(o, a["s2"], a["d2"], g)
        g_e2 = g.clone()
        g = self.d2a.backward(o, a["u2"], a["d2a"], g)
        g = self._up_bwd(g)
        g = self.d3.backward(o, a["s3"], a["d3"], g)
        g_e3 = g.clone()
        g = self.d3a.backward(o, a["u3"], a["d3a"], g)
        g = self._up_bwd(g)
        g = self.bt.backward(o, a["p3"], a["bt"], g)
        g_e3 += self._pool_bwd(g, a["e3"].shape[1], a["e3"].shape[2])
        g = self.e3.backward(o, a["e3a"], a["e3"], g_e3)
        g = self.e3a.backward(o, a["p2"], a["e3a"], g)
        g_e2 += self._pool_bwd(g, a["e2"].shape[1], a["e2"].shape[2])
        g = self.e2.backward(o, a["e2a"], a["e2"], g_e2)
        g = self.e2a.backward(o, a["p1"], a["e2a"], g)
        g_e1 += self._pool_bwd(g, a["e1"].shape[1], a["e1"].shape[2])
        g = self.e1.backward(o, a["e1a"], a["e1"], g_e1)
        self.e1a.backward(o, a["x"], a["e1a"], g, need_gx=False)

    def train_step(self, x, target, lr):
        """One Adam step on a batch; returns the loss (mean squared error)."""
        y = self.forward(x)
        P = y.shape[0] * y.shape[1] * y.shape[2]
        gy = torch.empty_like(y)
        loss = torch.zeros(1, dtype=torch.float32, device=y.device)
        self.ops.ctx._call("uwg_cnn_mse", int(P), 3, 3, _p(y), _p(target), _p(gy), _p(loss))
        self.backward(gy)
        self.step += 1
        for l in self.layers:
            l.adam(self.ops, self.step, lr)
        self.ops.check()
        return float(loss.item())

    def predict(self, x):
        y = self.forward(x)
        self._acts = None
        self.ops.check()
        return y


# ---------------------------------------------------------------------------
# Training data: random 2D Stokes problems solved by the library itself
# ---------------------------------------------------------------------------
def _grf(n, ell, gen, device):
    """Seeded Gaussian random field (Gaussian covariance, length ell) on an n^2
    periodic grid over the unit square, min-max scaled to [0, 1]."""
    noise = torch.randn((n, n), generator=gen, dtype=torch.float64).to(device)
    k = torch.fft.fftfreq(n, d=1.0 / n, device=device).double() * 2 * math.pi
    k2 = k[:, None] ** 2 + k[None, :] ** 2
    f = torch.fft.ifft2(torch.fft.fft2(noise) * torch.exp(-k2 * ell * ell / 4.0)).real
    return (f - f.min()) / (f.max() - f.min())


def _sample_grid(f, x):
    """Bilinear sample of an n^2 grid (node j at j/(n-1)) at points x [m, 2]."""
    n = f.shape[0]
    u = (x * (n - 1)).clamp(0, n - 1 - 1e-9)
    i0 = u.floor().long()
    t = u - i0
    v00 = f[i0[:, 1], i0[:, 0]]
    v10 = f[i0[:, 1], i0[:, 0] + 1]
    v01 = f[i0[:, 1] + 1, i0[:, 0]]
    v11 = f[i0[:, 1] + 1, i0[:, 0] + 1]
    return (v00 * (1 - t[:, 0]) * (1 - t[:, 1]) + v10 * t[:, 0] * (1 - t[:, 1]) + v01 * (1 - t[:, 0]) * t[:, 1]
            + v11 * t[:, 0] * t[:, 1])


def problem(seed, device):
    """Fields of one training problem: log10 viscosity = c (GRF - 1/2) with
    correlation length ~ U[0.05, 0.2] and contrast 10^c, c ~ U[3, 6]; 0-8
    circular inclusions of radius ~ U[0.03, 0.1] with density +-1."""
    rng = np.random.default_rng(seed)
    ell = rng.uniform(0.05, 0.2)
    c = rng.uniform(3.0, 6.0)
    k = int(rng.integers(0, 9))
    cen = rng.uniform(0.0, 1.0, (k, 2))
    rad = rng.uniform(0.03, 0.1, k)
    sgn = rng.choice([-1.0, 1.0], k)
    gen = torch.Generator().manual_seed(int(seed))
    T = _grf(256, ell, gen, device)

    def log_eta(x):
        return c * (_sample_grid(T, x) - 0.5)

    def rho(x):
        r = torch.zeros(x.shape[0], dtype=torch.float64, device=x.device)
        for j in range(k):
            inside = ((x[:, 0] - cen[j, 0]) ** 2 + (x[:, 1] - cen[j, 1]) ** 2) < rad[j] ** 2
            r = torch.where(inside, torch.full_like(r, sgn[j]), r)
        return r

    return log_eta, rho


def cell_centres(res, device):
    h = 1.0 / res
    c = (torch.arange(res, device=device, dtype=torch.float64) + 0.5) * h
    yy, xx = torch.meshgrid(c, c, indexing="ij")
    return torch.stack([xx.ravel(), yy.ravel()], 1)      # row-major cells, x fastest


def features(log_eta, rho, res, device):
    """Per-cell inputs: log10 viscosity / 3, buoyancy, and the hydrostatic
    pressure of the buoyancy column above the cell (mean-free, divided by its
    RMS); plus the scales of the problem: the reference viscosity 10^mean(log10
    eta) and the RMS of the hydrostatic pressure, by which targets are divided."""
    xc = cell_centres(res, device)
    le = log_eta(xc)
    r = rho(xc).reshape(res, res)
    # body force (0, -rho): dp/dy = -rho, p = 0 on top -> p(y) = sum of rho over the cells above
    hyd = torch.flip(torch.cumsum(torch.flip(r, [0]), 0), [0]) / res - 0.5 * r / res
    hyd = hyd - hyd.mean()
    s = float(torch.sqrt((hyd * hyd).mean()))
    s = s if s > 0.0 else 1.0
    f = torch.stack([le.reshape(res, res) / 3.0, r, hyd / s], 2)
    return f, (10.0 ** float(le.mean()), s)


def targets(u, p, res, scales):
    """Cell velocity (mean of the 4 nodes) and mean-free cell pressure, both
    divided by the hydrostatic scale, velocity also multiplied by the reference
    viscosity."""
    eta_ref, s = scales
    n = res + 1
    U = u.reshape(n, n, 2)
    uc = 0.25 * (U[:-1, :-1] + U[:-1, 1:] + U[1:, :-1] + U[1:, 1:])
    pc = (p - p.mean()).reshape(res, res, 1)
    return torch.cat([uc * (eta_ref / s), pc / s], 2)


def freeslip_mask(res):
    n = res + 1
    idx = np.arange(n * n)
    i, j = idx % n, idx // n
    m = np.zeros((n * n, 2), np.uint8)
    m[:, 0] = (i == 0) | (i == n - 1)
    m[:, 1] = (j == 0) | (j == n - 1)
    return torch.from_numpy(m.ravel())


class ProblemSet:
    """Assembles and solves the random problems on one 2D res^2 Q1/dQ0 context
    with ppc particles per element (seeded layout)."""

    def __init__(self, res=128, ppc=20):
        from ._core import Context
        self.res, self.ppc = res, ppc
        self.ctx = Context(2, (res, res), (0.0, 0.0), (1.0, 1.0))
        self.ctx.set_bcs(freeslip_mask(res))

    def assemble(self, seed):
        from ._core import rng_seed
        ctx = self.ctx
        log_eta, rho = problem(seed, ctx.device)
        x, owner, off, lst, _ = ctx.layout_random(self.ppc, rng_seed(int(seed) % 100000 + 1))
        eta = torch.pow(10.0, log_eta(x)).contiguous()
        body = torch.zeros_like(x)
        body[:, 1] = -rho(x)
        ip_xi = ctx.pic_map(x, off, lst)
        ip_w = ctx.dvc_weights(off, ip_xi)
        ctx.assemble(off, lst, ip_xi, ip_w, eta, body.contiguous())
        f, scales = features(log_eta, rho, self.res, ctx.device)
        return f, scales

    def solve(self, mixed, p0=None, p_dir=None, rtol=1e-8, coarse_agg=0):
        """Solve the assembled problem; p0: initial pressure, p_dir: first search
        direction of the Schur FGMRES (both device tensors, or None); coarse_agg > 0:
        the coarse-level correction of the Schur FGMRES with that aggregate size."""
        ctx = self.ctx
        u = ctx.zeros(ctx.n_vdof)
        p = ctx.zeros(ctx.n_pdof) if p0 is None else p0.reshape(-1).to(torch.float64).contiguous().clone()
        d = None if p_dir is None else p_dir.reshape(-1).to(torch.float64).contiguous()
        st = ctx.solve(u, p, mixed=int(mixed), rtol=rtol, inner_rtol=1e-10, outer_rtol=1e-9, smooth_steps=2,
                       restart=120, schur_pc=1, max_outer=500, zero_guess=0 if p0 is not None else 1,
                       p_dir=None if d is None else d.data_ptr(), coarse_agg=int(coarse_agg))
        return u, p, st


def generate(ps, seeds, rtol=1e-8):
    """Inputs [n, res, res, 2] and targets [n, res, res, 3] (FP32, device)."""
    res = ps.res
    X = torch.empty((len(seeds), res, res, 3), dtype=torch.float32, device=ps.ctx.device)
    Y = torch.empty((len(seeds), res, res, 3), dtype=torch.float32, device=ps.ctx.device)
    for i, s in enumerate(seeds):
        f, scales = ps.assemble(s)
        u, p, st = ps.solve(1, rtol=rtol)
        X[i] = f.float()
        Y[i] = targets(u, p, res, scales).float()
    return X, Y


def train(net, X, Y, epochs=20, batch=8, lr=1e-3, lr_final=1e-4, seed=0, log=None):
    """Adam with an exponentially decaying learning rate on targets scaled per
    channel by their standard deviation over the training set."""
    n = X.shape[0]
    net.scale = Y.reshape(-1, 3).std(dim=0).clamp_min(1e-12).float()
    Y = (Y / net.scale).contiguous()
    gen = torch.Generator().manual_seed(seed)
    steps = epochs * ((n + batch - 1) // batch)
    k = 0
    losses = []
    for ep in range(epochs):
        perm = torch.randperm(n, generator=gen)
        tot = 0.0
        for b0 in range(0, n - batch + 1, batch):
            idx = perm[b0: b0 + batch].to(X.device)
            lr_k = lr * (lr_final / lr) ** (k / max(steps - 1, 1))
            tot += net.train_step(X[idx].to(_BF).contiguous(), Y[idx].contiguous(), lr_k)
            k += 1
        losses.append(tot / max(n // batch, 1))
        if log:
            log(ep, losses[-1])
    return losses


def predict_pressure(net, f, scales):
    """Cell pressure guess (mean-free) for one problem's feature grid."""
    y = net.predict(f[None].to(_BF).contiguous())
    p = y[0, :, :, 2].reshape(-1).double() * (float(net.scale[2]) * scales[1])
    return p - p.mean()


def solve_with_warm_start(ps, net, f, scales, rtol=1e-8, mode="direction", coarse_agg=0):
    """Mixed-precision solve using the network's pressure -- as the first search
    direction of the Schur FGMRES (mode "direction": the iteration's least-squares
    step weighs it) or as the initial guess (mode "guess") -- and the plain FP64
    solve if that does not reach rtol.  coarse_agg > 0 adds the coarse-level
    correction of the Schur FGMRES.  Returns (u, p, stats, fell_back)."""
    p0 = predict_pressure(net, f, scales)
    try:
        if not bool(torch.isfinite(p0).all()):
            raise FloatingPointError("non-finite network output")
        if mode == "guess":
            u, p, st = ps.solve(1, p0=p0, rtol=rtol, coarse_agg=coarse_agg)
        else:
            u, p, st = ps.solve(1, p_dir=p0, rtol=rtol, coarse_agg=coarse_agg)
        if st["residual"] <= rtol:
            return u, p, st, False
    except (FloatingPointError, _native.UwgError):
        pass
    u, p, st = ps.solve(0, rtol=rtol)
    return u, p, st, True
