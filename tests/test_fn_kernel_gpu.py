"""The compiled function-graph evaluation (one kernel per graph, uwg_fn_eval)
against the tensor evaluation of the same graphs: constants, coordinates,
swarm variables of several dtypes, arithmetic, math functions, comparisons
and logic, branching.map / branching.conditional, vectors, dot, SafeMaths,
and the errors the reference raises (a key with no mapping and no default,
no true clause, a non-finite SafeMaths value).  Values agree to a few ulp
(both sides call CUDA's math functions)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


class _Var:
    def __init__(self, t):
        self.t = t

    def _device_data(self):
        return self.t


def _setup(n=4000, npart=1500, seed=0):
    from underworld2_gb300 import function as fn
    from underworld2_gb300._core import Context
    c = Context(2, (8, 8), (0.0, 0.0), (1.0, 1.0))
    rng = np.random.default_rng(seed)
    dev = torch.device("cuda")
    pid = torch.tensor(rng.integers(0, npart, n), dtype=torch.int32, device=dev)
    xy = torch.tensor(rng.uniform(0.0, 1.0, (n, 2)), device=dev)
    ctx = fn.EvalContext(pid.long(), lambda: xy, dev, lib_ctx=c, pid32=pid)
    mat = fn._SwarmVar(_Var(torch.tensor(rng.integers(0, 3, (npart, 1)), dtype=torch.int32, device=dev)))
    T = fn._SwarmVar(_Var(torch.tensor(rng.uniform(0.0, 1.0, (npart, 1)), device=dev)))
    T32 = fn._SwarmVar(_Var(torch.tensor(rng.uniform(0.0, 1.0, (npart, 2)), dtype=torch.float32, device=dev)))
    return fn, ctx, mat, T, T32, npart


def _both(fn, f, ctx, ncomp=None):
    k = fn._eval_kernel(f, ctx, ncomp)
    assert k is not None, "graph not compiled"
    t = f.evaluate_at(ctx).to(torch.float64)
    if ncomp is not None and t.shape[1] == 1 and ncomp > 1:
        t = t.expand(-1, ncomp)
    return k.cpu().numpy(), t.cpu().numpy()


def test_arithmetic_math_and_logic(gpu):
    fn, ctx, mat, T, T32, _ = _setup()
    x, y = fn.input()[0], fn.input()[1]
    graphs = [
        fn.math.exp(-11.5 * T) * (1.0 + fn.math.sin(3.0 * x) * fn.math.cos(2.0 * y)) / fn.math.sqrt(fn.math.abs(T) + 1.0),
        fn.misc.max(T, 0.3) - fn.misc.min(x, y) + fn.math.pow(T + 1.0, 2.5) - T32[1],
        fn.math.log10(T + 2.0) + fn.math.tanh(x - y) + fn.math.erf(T) + fn.math.atan(y) - fn.math.log(x + 1.0),
        (x > 0.5) & (y < 0.5) | (T >= 0.2) ^ (T32[0] <= 0.7),
        fn.math.dot((x, y), (T, 2.0)),
        -(x * y) + 3.0,
    ]
    for f in graphs:
        k, t = _both(fn, f, ctx)
        np.testing.assert_allclose(k, t, rtol=1e-14, atol=1e-300)


def test_map_conditional_and_vectors(gpu):
    fn, ctx, mat, T, T32, _ = _setup()
    x = fn.input()[0]
    visc = fn.branching.map(fn_key=mat, mapping={0: 1.0, 1: 100.0, 2: fn.math.exp(-2.0 * T)})
    dens = fn.branching.map(fn_key=mat, mapping={1: 1.0}, fn_default=0.25 * x)
    cond = fn.branching.conditional([(x < 0.3, 1.0), (visc > 10.0, visc * 2.0), (True, T)])
    body = dens * (0.0, -1.0)
    for f, nc in ((visc, None), (dens, None), (cond, None), (body, 2), (fn.Function.convert((T, x, 1.0)), 3)):
        k, t = _both(fn, f, ctx, nc)
        np.testing.assert_allclose(k, t, rtol=1e-14, atol=1e-300)


def test_scatter_into_particle_order(gpu):
    """With an output array the kernel writes each point's value into its particle's row."""
    fn, ctx, mat, T, T32, npart = _setup(n=1500, npart=1500)
    perm = torch.randperm(1500, device="cuda")
    ctx.pid, ctx.pid32 = perm, perm.to(torch.int32)
    f = fn.math.exp(-2.0 * T) + fn.input()[1]
    out = torch.zeros((npart, 1), dtype=torch.float64, device="cuda")
    assert fn._eval_kernel(f, ctx, 1, out) is not None
    ref = torch.zeros_like(out)
    ref[ctx.pid] = f.evaluate_at(ctx)
    np.testing.assert_allclose(out.cpu().numpy(), ref.cpu().numpy(), rtol=1e-14)


def test_errors_match_the_tensor_path(gpu):
    fn, ctx, mat, T, T32, _ = _setup()
    nodef = fn.branching.map(fn_key=mat, mapping={0: 1.0, 1: 2.0})   # key 2 occurs, no default
    with pytest.raises(RuntimeError, match="map"):
        fn._eval_kernel(nodef, ctx)
    with pytest.raises(RuntimeError, match=r"key \(2\)"):
        nodef.evaluate_at(ctx)
    nocase = fn.branching.conditional([(fn.input()[0] < -1.0, 1.0)])
    with pytest.raises(RuntimeError):
        fn._eval_kernel(nocase, ctx)
    safe = fn.exception.SafeMaths(fn.math.log(T - 2.0))
    with pytest.raises(RuntimeError):
        fn._eval_kernel(safe, ctx)
    ok = fn.exception.SafeMaths(fn.math.log(T + 2.0))
    k, t = _both(fn, ok, ctx)
    np.testing.assert_allclose(k, t, rtol=1e-14)


def test_unsupported_nodes_fall_back(gpu):
    """A node kind outside the program (a polygon shape) leaves evaluation to the tensor path."""
    fn, ctx, mat, T, T32, _ = _setup()
    poly = fn.shape.Polygon(np.array([[0.1, 0.1], [0.9, 0.2], [0.5, 0.8]]))
    assert fn._eval_kernel(poly * T, ctx) is None
