"""The function graph (underworld.function subset) evaluated on the CPU: math,
misc, tensor, shape, view, exception and rheology functions against numpy,
with the reference docstrings' known answers where they give one
(P/function/math.py, shape.py:44-56)."""
import math

import numpy as np
import pytest
import torch

import underworld2_gb300 as uw
from underworld2_gb300 import function as fn


def test_math_functions_match_numpy():
    x = np.array([[0.1], [0.35], [0.8]])
    cases = {"cos": np.cos, "sin": np.sin, "tan": np.tan, "acos": np.arccos, "asin": np.arcsin, "atan": np.arctan,
             "cosh": np.cosh, "sinh": np.sinh, "tanh": np.tanh, "asinh": np.arcsinh, "atanh": np.arctanh,
             "exp": np.exp, "log": np.log, "log2": np.log2, "log10": np.log10, "sqrt": np.sqrt, "abs": np.abs}
    for name, ref in cases.items():
        np.testing.assert_allclose(getattr(fn.math, name)().evaluate(x), ref(x), rtol=1e-15, atol=0, err_msg=name)
    np.testing.assert_allclose(fn.math.acosh().evaluate(x + 1.0), np.arccosh(x + 1.0), rtol=1e-15)
    np.testing.assert_allclose(fn.math.erf().evaluate(x), [[math.erf(v)] for v in x[:, 0]], rtol=1e-15)
    np.testing.assert_allclose(fn.math.erfc().evaluate(x), [[math.erfc(v)] for v in x[:, 0]], rtol=1e-15)
    # docstring: sin at (0, pi/4, 2 pi) as one 3-vector input
    np.testing.assert_allclose(fn.math.sin().evaluate((0.0, math.pi / 4.0, 2.0 * math.pi)),
                               [[0.0, 0.5 * math.sqrt(2.0), 0.0]], atol=1e-15)
    np.testing.assert_allclose(fn.math.pow(fn.input(), 3.0).evaluate(x), x ** 3, rtol=1e-15)
    np.testing.assert_allclose(fn.math.dot(fn.input(), fn.input()).evaluate(np.array([[1.0, 2.0, 3.0]])), [[14.0]])


def test_misc_min_max_and_comparisons():
    x = np.array([[0.2], [0.7]])
    np.testing.assert_array_equal(fn.misc.max(fn.input(), 0.5).evaluate(x), [[0.5], [0.7]])
    np.testing.assert_array_equal(fn.misc.min(fn.input(), 0.5).evaluate(x), [[0.2], [0.5]])
    r = (fn.input() > 0.5).evaluate(x)
    assert r.dtype == bool and r.tolist() == [[False], [True]]


class _Full(fn.Function):
    """A full (row-major) tensor value for the tensor-function tests."""
    _kind = "tensor"

    def __init__(self, t):
        self.t = t

    def _eval(self, ctx):
        return torch.as_tensor(self.t, dtype=torch.float64, device=ctx.device)


@pytest.mark.parametrize("dim", [2, 3])
def test_tensor_functions(dim):
    rng = np.random.default_rng(dim)
    F = rng.standard_normal((5, dim, dim))
    full = _Full(F.reshape(5, -1))
    S = 0.5 * (F + F.transpose(0, 2, 1))
    order = [(0, 0), (1, 1), (0, 1)] if dim == 2 else [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
    sym = fn.tensor.symmetric(full)
    np.testing.assert_allclose(sym.evaluate(np.zeros((5, dim))), np.stack([S[:, i, j] for i, j in order], 1),
                               rtol=1e-15)
    A = 0.5 * (F - F.transpose(0, 2, 1))
    np.testing.assert_allclose(fn.tensor.antisymmetric(full).evaluate(np.zeros((5, dim))), A.reshape(5, -1),
                               rtol=1e-15, atol=1e-16)
    np.testing.assert_allclose(fn.tensor.second_invariant(full).evaluate(np.zeros((5, dim))),
                               np.sqrt(0.5 * (F * F).sum((1, 2)))[:, None], rtol=1e-15)
    np.testing.assert_allclose(fn.tensor.second_invariant(sym).evaluate(np.zeros((5, dim))),
                               np.sqrt(0.5 * (S * S).sum((1, 2)))[:, None], rtol=1e-14)
    D = S - np.einsum("nii->n", S)[:, None, None] / dim * np.eye(dim)
    np.testing.assert_allclose(fn.tensor.deviatoric(sym).evaluate(np.zeros((5, dim))),
                               np.stack([D[:, i, j] for i, j in order], 1), rtol=1e-14, atol=1e-15)
    # a scalar times a symmetric tensor stays a symmetric tensor
    np.testing.assert_allclose(fn.tensor.second_invariant(2.0 * sym).evaluate(np.zeros((5, dim))),
                               2.0 * np.sqrt(0.5 * (S * S).sum((1, 2)))[:, None], rtol=1e-14)
    with pytest.raises(ValueError):
        fn.tensor.symmetric(fn.input())
    with pytest.raises(ValueError):
        fn.tensor.deviatoric(full)


def test_polygon_docstring_and_random_points():
    tri = np.array([(0.0, 0.0), (0.5, 1.0), (1.0, 0.0)])
    poly = fn.shape.Polygon(tri)
    assert poly.evaluate(np.array([(0.0, 0.9), (0.5, 0.5), (0.9, 0.2)])).tolist() == [[False], [True], [False]]
    sq = fn.shape.Polygon(np.array([(0.2, 0.2), (0.8, 0.2), (0.8, 0.7), (0.2, 0.7)]))
    pts = np.random.default_rng(1).uniform(0.0, 1.0, (400, 2))
    inside = (pts[:, 0] > 0.2) & (pts[:, 0] < 0.8) & (pts[:, 1] > 0.2) & (pts[:, 1] < 0.7)
    np.testing.assert_array_equal(sq.evaluate(pts)[:, 0], inside)
    with pytest.raises(TypeError):
        fn.shape.Polygon(np.array([(0.0, 0.0), (1.0, 1.0)]))


def test_view_exception_rheology():
    mm = fn.view.min_max(fn.input()[0] * 2.0)
    mm.evaluate(np.array([[0.1], [0.4], [-0.3]]))
    assert mm.min_global() == pytest.approx(-0.6) and mm.max_global() == pytest.approx(0.8)
    with pytest.raises(RuntimeError):
        fn.exception.SafeMaths(fn.math.sqrt(fn.input())).evaluate(np.array([[-1.0]]))
    stress = _Full(np.array([[3.0, 0.0, 0.0, -3.0], [0.1, 0.0, 0.0, -0.1]]))
    sym = fn.tensor.symmetric(stress)
    lim = fn.rheology.stress_limiting_viscosity(sym, 1.0, 10.0)
    np.testing.assert_allclose(lim.evaluate(np.zeros((2, 2))), [[10.0 / 3.0], [10.0]], rtol=1e-15)


def test_branching():
    x = np.array([[0.0], [1.0], [2.0]])
    m = fn.branching.map(fn_key=fn.input()[0], mapping={0: 10.0, 1: 20.0}, fn_default=30.0)
    np.testing.assert_array_equal(m.evaluate(x), [[10.0], [20.0], [30.0]])
    c = fn.branching.conditional([(fn.input()[0] < 0.5, -1.0), (True, 1.0)])
    np.testing.assert_array_equal(c.evaluate(x), [[-1.0], [1.0], [1.0]])


def test_view_count_and_custom_exception():
    """P/function/view.py:385-440 and P/function/exception.py:69-140 docstring behaviour."""
    import underworld2_gb300.function as fn
    c = fn.view.count(fn.input())
    c.evaluate(5.0)
    assert c.count() == 1
    for _ in range(3):
        c.evaluate(5.0)
    assert c.count() == 4
    c.reset()
    c.evaluate(5.0)
    c.evaluate(5.0)
    assert c.count() == 2
    c.evaluate(np.zeros((7, 2)))          # one count per point
    assert c.count() == 9
    one = fn.misc.constant(1.0)
    np.testing.assert_array_equal(fn.exception.CustomException(one, one < 2.0).evaluate(), [[1.0]])
    with pytest.raises(RuntimeError, match="evaluated to False"):
        fn.exception.CustomException(one, one > 2.0).evaluate()
    with pytest.raises(RuntimeError, match=r"\( 5 \)"):
        fn.exception.CustomException(one, one * 5.0 > 20.0, one * 5.0).evaluate()
