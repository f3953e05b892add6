"""Known answers from the reference's function-module docstrings, restated as
tests (CPU; no mesh or swarm needed).  Each case cites the docstring it
follows; the asserted values and types are the ones printed there."""
import numpy as np
import pytest

from underworld2_gb300 import function as fn


def test_constants_keep_their_type():
    """P/function/misc.py:27-46 and P/function/_function.py:210-214."""
    a = fn.misc.constant(3).evaluate(0.)
    assert a.dtype == np.int32 and a.tolist() == [[3]]
    a = fn.misc.constant((3, 2, 1)).evaluate(0.)
    assert a.dtype == np.int32 and a.tolist() == [[3, 2, 1]]
    a = fn.misc.constant(3.).evaluate(0.)
    assert a.dtype == np.float64 and a.tolist() == [[3.0]]
    a = fn.misc.constant((3., 2., 1.)).evaluate(0.)
    assert a.dtype == np.float64 and a.tolist() == [[3.0, 2.0, 1.0]]
    a = fn.misc.constant(True).evaluate(0.)
    assert a.dtype == bool and a.tolist() == [[True]]
    a = fn.misc.constant((True, False, True)).evaluate(0.)
    assert a.dtype == bool and a.tolist() == [[True, False, True]]
    a = fn.Function.convert(3).evaluate(0.)
    assert a.dtype == np.int32 and a.tolist() == [[3]]


def test_vector_conversion():
    """P/function/_function.py:220-227."""
    fn1, fn2, fn3 = fn.input(), 10. * fn.input(), 100. * fn.input()
    np.testing.assert_array_equal(fn.Function.convert((fn1, fn2, fn3)).evaluate([3.]), [[3., 30., 300.]])


def test_arithmetic_on_constants():
    """P/function/_function.py:282-437."""
    two, three, four = fn.misc.constant(2.), fn.misc.constant(3.), fn.misc.constant(4.)
    assert np.allclose((three + four).evaluate(0.), [[7.]])
    assert np.allclose((three - four).evaluate(0.), [[-1.]])
    assert np.allclose((5. - four).evaluate(0.), [[1.]])
    assert np.allclose((-four).evaluate(0.), [[-4.]])
    assert np.allclose((three * four).evaluate(0.), [[12.]])
    assert np.allclose((four / two).evaluate(0.), [[2.]])
    assert np.allclose((two ** four).evaluate(0.), [[16.]])


def test_comparisons_and_logic():
    """P/function/_function.py:455-620."""
    two, four = fn.misc.constant(2.), fn.misc.constant(4.)
    for f, expect in (((two < four), True), ((two <= two), True), ((two > four), False), ((two >= two), True)):
        a = f.evaluate()
        assert a.dtype == bool and a.tolist() == [[expect]]
    t, f_ = fn.misc.constant(True), fn.misc.constant(False)
    assert (t & f_).evaluate().tolist() == [[False]]
    assert (t | f_).evaluate().tolist() == [[True]]
    assert (t ^ f_).evaluate().tolist() == [[True]]
    assert (t ^ t).evaluate().tolist() == [[False]]


def test_component_and_input():
    """P/function/_function.py:645-649, 1264-1281."""
    assert np.allclose(fn.misc.constant((2., 3., 4.))[1].evaluate(0.), [[3.]])
    assert np.allclose(fn.input().evaluate((1., 2., 3.)), [1., 2., 3.])
    density = 1. - 0.01 * fn.input()[1]
    assert np.allclose(density.evaluate((0.1, 0.4)), density.evaluate((0.9, 0.4)))


def test_min_max_against_conditional():
    """P/function/misc.py:150-166."""
    testpoints = np.array([[0.0], [0.2], [0.4], [0.6], [0.8], [1.01], [1.2], [1.4], [1.6], [1.8], [2.0]])
    x = fn.input()[0]
    x_minus_one, one_minus_x = x - 1., 1. - x
    fn_max = fn.misc.max(one_minus_x, x_minus_one)
    fn_min = fn.misc.min(one_minus_x, x_minus_one)
    cmax = fn.branching.conditional(((x <= 1., one_minus_x), (x > 1., x_minus_one)))
    cmin = fn.branching.conditional(((x >= 1., one_minus_x), (x < 1., x_minus_one)))
    assert np.allclose(fn_max.evaluate(testpoints), cmax.evaluate(testpoints))
    assert np.allclose(fn_min.evaluate(testpoints), cmin.evaluate(testpoints))


def test_view_count():
    """P/function/view.py:396-423."""
    fn_count = fn.view.count(fn.input())
    fn_count.evaluate(5.)
    assert fn_count.count() == 1
    for _ in range(3):
        fn_count.evaluate(5.)
    assert fn_count.count() == 4
    fn_count.reset()
    fn_count.evaluate(5.)
    fn_count.evaluate(5.)
    assert fn_count.count() == 2


def test_exceptions():
    """P/function/exception.py:38-50 (SafeMaths on 1/0) and 95-115 (CustomException)."""
    one, zero = fn.misc.constant(1.), fn.misc.constant(0.)
    with pytest.raises(RuntimeError):
        fn.exception.SafeMaths(one / zero).evaluate()
    assert fn.exception.CustomException(one, (one < 2.)).evaluate().tolist() == [[1.0]]
    with pytest.raises(RuntimeError):
        fn.exception.CustomException(one, (one > 2.)).evaluate()
    with pytest.raises(RuntimeError):
        fn.exception.CustomException(one, (one * 5. > 20.), one * 5.).evaluate()


def test_conditional_integral_of_unit_disc():
    """P/function/branching.py:189-197: the indicator of the unit disc,
    integrated over [-1, 1]^2 on 16 x 16 Q1 elements, is pi within 1e-2."""
    import underworld2_gb300 as uw
    mesh = uw.mesh.FeMesh_Cartesian(elementRes=(16, 16), minCoord=(-1.0, -1.0), maxCoord=(1.0, 1.0))
    circleFn = fn.coord()[0] ** 2 + fn.coord()[1] ** 2
    fn_conditional = fn.branching.conditional([(circleFn < 1.0, 1.0), (True, 0.0)])
    assert np.allclose(np.pi, uw.utils.Integral(fn_conditional, mesh).evaluate(), rtol=1e-2)


def test_view_min_max():
    """P/function/view.py:52-121: min_max records the extremes over every
    evaluation; a non-scalar function needs fn_norm; fn_auxiliary is recorded
    at the extremes (P/function/view.py:150-245)."""
    fn_simple = fn.input()[0] * 2.0
    mm = fn.view.min_max(fn_simple)
    assert mm.evaluate(5.0).tolist() == [[10.0]] and mm.min_global() == 10.0 and mm.max_global() == 10.0
    assert mm.evaluate(-3.0).tolist() == [[-6.0]] and mm.min_global() == -6.0 and mm.max_global() == 10.0
    assert fn_simple.evaluate(3000.0).tolist() == [[6000.0]] and mm.max_global() == 10.0
    fn_vec = fn.input() * (1.0, 1.0)
    with pytest.raises(RuntimeError, match="does not return scalar results"):
        fn.view.min_max(fn_vec).evaluate(2.0)
    vm = fn.view.min_max(fn_vec, fn_norm=fn.math.dot(fn_vec, fn_vec))
    assert vm.evaluate(2.0).tolist() == [[2.0, 2.0]] and vm.max_global() == 8.0
    assert vm.evaluate(-1.0).tolist() == [[-1.0, -1.0]] and vm.min_global() == 2.0 and vm.max_global() == 8.0
    pts = np.array([[0.3, 0.1], [-0.2, 0.5], [0.05, 0.9], [0.7, -0.4]])
    am = fn.view.min_max(fn.math.abs(fn.input()[0]), fn_auxiliary=fn.input())
    am.evaluate(pts)
    np.testing.assert_array_equal(am.min_global_auxiliary(), [[0.05, 0.9]])
    np.testing.assert_array_equal(am.max_global_auxiliary(), [[0.7, -0.4]])
    am.reset()
    assert am.min_global() == float("inf") and am.min_global_auxiliary() is None


def test_polygon_shape():
    """P/function/shape.py:50-64: points inside a triangle."""
    polyfn = fn.shape.Polygon(np.array([(0.0, 0.0), (0.5, 1.0), (1.0, 0.0)]))
    res = polyfn.evaluate(np.array([(0.0, 0.9), (0.5, 0.5), (0.9, 0.2)]))
    assert res.dtype == bool and res.tolist() == [[False], [True], [False]]


def test_convert_identity_integrate_and_vector_input():
    """P/function/_function.py:209-226, 793-799, 841-853: convert is the identity on
    a Function and passes None; Function.integrate over a mesh; a unary math
    function applies per component of a vector input; empty inputs give empty
    results."""
    import math as sysmath
    import underworld2_gb300 as uw
    fn_const = fn.Function.convert(3)
    assert fn_const is fn.Function.convert(fn_const) and fn.Function.convert(None) is None
    mesh = uw.mesh.FeMesh_Cartesian(minCoord=(0.0, 0.0), maxCoord=(1.0, 2.0))
    assert np.allclose(fn.misc.constant(2.0).integrate(mesh)[0], 4)
    assert np.allclose((fn.misc.constant(2.0) * (0.5, 1.0)).integrate(mesh), [2, 4])
    sinfn = fn.math.sin()
    assert np.allclose(sinfn.evaluate(sysmath.pi / 4.0), [[0.5 * sysmath.sqrt(2.0)]])
    assert np.allclose(sinfn.evaluate((0.0, sysmath.pi / 4.0, 2.0 * sysmath.pi)), [[0.0, 0.5 * sysmath.sqrt(2.0), 0.0]])
    var = uw.mesh.MeshVariable(uw.mesh.FeMesh_Cartesian(), 1)
    assert var.evaluate(np.zeros((0, 2))).shape == (0, 1)
    assert var.evaluate(var.mesh.specialSets["Empty"]).shape == (0, 1)
