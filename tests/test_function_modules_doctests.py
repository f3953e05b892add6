"""Docstring known answers of uw.function.math, misc and branching
(P/function/math.py, P/function/misc.py, P/function/branching.py), with the
argument checks those modules make.  CPU: coordinate inputs and mesh-only
integrals."""
import math as sysmath

import numpy as np
import pytest

import underworld2_gb300 as uw

fn = uw.function

_MATH = [("cos", 0.1234, sysmath.cos), ("sin", 0.1234, sysmath.sin), ("tan", 0.1234, sysmath.tan),
         ("acos", 0.1234, sysmath.acos), ("asin", 0.1234, sysmath.asin), ("atan", 0.1234, sysmath.atan),
         ("cosh", 0.1234, sysmath.cosh), ("sinh", 0.1234, sysmath.sinh), ("tanh", 0.1234, sysmath.tanh),
         ("acosh", 5.1234, sysmath.acosh), ("asinh", 5.1234, sysmath.asinh), ("atanh", 0.1234, sysmath.atanh),
         ("exp", 0.1234, sysmath.exp), ("log", 0.1234, sysmath.log), ("log2", 0.1234, lambda v: sysmath.log(v, 2)),
         ("log10", 0.1234, sysmath.log10), ("sqrt", 0.1234, sysmath.sqrt), ("erf", 0.1234, sysmath.erf),
         ("erfc", 0.1234, sysmath.erfc), ("abs", -0.1234, sysmath.fabs)]


@pytest.mark.parametrize("name,x,ref", _MATH, ids=[m[0] for m in _MATH])
def test_math_functions(name, x, ref):
    """P/function/math.py:34-648: each function of the input against Python's math."""
    v = getattr(fn.math, name)().evaluate(x)
    assert v.shape == (1, 1) and v.dtype == np.float64
    assert np.allclose(v, ref(x))


def test_math_pow_and_dot():
    """P/function/math.py:679-727."""
    assert np.allclose(fn.math.pow(fn.input(), 3.0).evaluate(2.0), sysmath.pow(2.0, 3.0))
    a, b = (2.0, 3.0, 4.0), (5.0, 6.0, 7.0)
    assert np.allclose(fn.math.dot(a, b).evaluate(0.0), np.dot(a, b))


def test_constant_types():
    """P/function/misc.py:28-47: a constant keeps its type."""
    out = [fn.misc.constant(v).evaluate(0.0) for v in (3, (3, 2, 1), 3.0, (3.0, 2.0, 1.0), True, (True, False, True))]
    assert [o.dtype for o in out] == [np.int32, np.int32, np.float64, np.float64, bool, bool]
    assert [o.tolist() for o in out] == [[[3]], [[3, 2, 1]], [[3.0]], [[3.0, 2.0, 1.0]], [[True]],
                                         [[True, False, True]]]


def test_constant_value_checks():
    """P/function/misc.py:59-126: values are bools, ints or floats, or non-empty
    iterables homogeneous in one of them; a reset keeps the type and size."""
    c = fn.misc.constant(3)
    c.value = 5
    assert c.evaluate(0.0).tolist() == [[5]]
    with pytest.raises(TypeError, match="identical type"):
        c.value = 3.0
    v = fn.misc.constant((1.0, 2.0))
    with pytest.raises(TypeError, match="identical size"):
        v.value = (1.0, 2.0, 3.0)
    v.value = (4.0, 5.0)
    assert v.evaluate(0.0).tolist() == [[4.0, 5.0]]
    with pytest.raises(ValueError, match="does not appear to be valid"):
        fn.misc.constant(object())
    with pytest.raises(ValueError, match="zero size"):
        fn.misc.constant(())
    with pytest.raises(ValueError, match="'int', 'float' or 'bool'"):
        fn.misc.constant("abc")
    with pytest.raises(ValueError, match="homogeneous"):
        fn.misc.constant((1, 2.0))
    # conversion of a mixed tuple gives a float vector, as the reference's vector of basis functions does
    mixed = fn.Function.convert((1, 2.0))
    assert mixed.evaluate(0.0).dtype == np.float64 and mixed.evaluate(0.0).tolist() == [[1.0, 2.0]]


def test_misc_min_max():
    """P/function/misc.py:140-166: min/max against the equivalent conditionals."""
    pts = np.array([[0.0], [0.2], [0.4], [0.6], [0.8], [1.01], [1.2], [1.4], [1.6], [1.8], [2.0]])
    x = fn.input()[0]
    fn_max = fn.misc.max(1.0 - x, x - 1.0)
    fn_min = fn.misc.min(1.0 - x, x - 1.0)
    cmax = fn.branching.conditional(((x <= 1.0, 1.0 - x), (x > 1.0, x - 1.0)))
    cmin = fn.branching.conditional(((x >= 1.0, 1.0 - x), (x < 1.0, x - 1.0)))
    assert np.allclose(fn_max.evaluate(pts), cmax.evaluate(pts))
    assert np.allclose(fn_min.evaluate(pts), cmin.evaluate(pts))


def test_conditional_unit_circle():
    """P/function/branching.py:189-197: the unit disc's area on a 16 x 16 mesh."""
    mesh = uw.mesh.FeMesh_Cartesian(elementRes=(16, 16), minCoord=(-1.0, -1.0), maxCoord=(1.0, 1.0))
    circle = fn.coord()[0] ** 2 + fn.coord()[1] ** 2
    cond = fn.branching.conditional([(circle < 1.0, 1.0), (True, 0.0)])
    assert np.allclose(np.pi, uw.utils.Integral(cond, mesh).evaluate(), rtol=1e-2)


def test_branching_argument_checks():
    """P/function/branching.py:102-140, 199-215, and the evaluation errors of
    Map.cpp:118-124 and Conditional.cpp:117."""
    x = fn.input()[0]
    with pytest.raises(ValueError, match="specify a mapping"):
        fn.branching.map(fn_key=x, mapping=None)
    with pytest.raises(TypeError, match="dict"):
        fn.branching.map(fn_key=x, mapping=[(0, 1.0)])
    with pytest.raises(ValueError, match="key function"):
        fn.branching.map(mapping={0: 1.0})
    with pytest.raises(ValueError, match="unsigned integers"):
        fn.branching.map(fn_key=x, mapping={-1: 1.0})
    with pytest.raises(ValueError, match="unsigned integers"):
        fn.branching.map(fn_key=x, mapping={1.5: 1.0})
    with pytest.raises(ValueError, match="'None' is not valid"):
        fn.branching.map(fn_key=x, mapping={0: None})
    with pytest.raises(TypeError, match="'list' or 'tuple'"):
        fn.branching.conditional("abc")
    with pytest.raises(TypeError, match="Clauses within"):
        fn.branching.conditional([1])
    with pytest.raises(ValueError, match="length 2"):
        fn.branching.conditional([(True, 1.0, 2.0)])
    with pytest.raises(RuntimeError, match="Reached end of conditional"):
        fn.branching.conditional([(x > 5.0, 1.0)]).evaluate(0.0)
    with pytest.raises(RuntimeError, match=r"key \(3\)"):
        fn.branching.map(fn_key=fn.misc.constant(3), mapping={0: 1.0}).evaluate(0.0)
    assert fn.branching.map(fn_key=fn.misc.constant(3), mapping={0: 1.0}, fn_default=2.0).evaluate(0.0).tolist() \
        == [[2.0]]


def test_numpy_values_convert():
    """Function.convert turns numpy arrays and scalars into constants, as the
    reference's conversion through misc.constant does (P/function/_function.py:230-260)."""
    assert fn.Function.convert(np.array([1.0, 2.0])).evaluate(0.0).tolist() == [[1.0, 2.0]]
    assert fn.Function.convert(np.bool_(True)).evaluate(0.0).dtype == bool
    assert (fn.input()[0] * np.array((0.0, -1.0))).evaluate(2.0).tolist() == [[0.0, -2.0]]


def test_exception_and_rheology_argument_checks():
    """P/function/exception.py:57-60,131-145 and P/function/rheology.py:94-108:
    missing functions are refused with ValueError."""
    with pytest.raises(ValueError, match="'fn'"):
        fn.exception.SafeMaths(None)
    with pytest.raises(ValueError):
        fn.exception.CustomException(None, True)
    with pytest.raises(ValueError):
        fn.exception.CustomException(1.0, None)
    for args, name in (((None, 1.0, 1.0), "fn_stress"), ((1.0, None, 1.0), "fn_stresslimit"),
                       ((1.0, 1.0, None), "fn_inputviscosity")):
        with pytest.raises(ValueError, match=name):
            fn.rheology.stress_limiting_viscosity(*args)
    one = fn.misc.constant(1.0)
    with pytest.raises(RuntimeError, match=r"\( 5 \)"):
        fn.exception.CustomException(one, one * 5.0 > 20.0, one * 5.0).evaluate()


def test_evaluate_global_single_process():
    """P/function/_function.py:654-759 on one process: the root's result is the
    plain evaluation; object inputs are refused."""
    x = fn.input()
    pts = np.array([[0.1, 0.2], [0.3, 0.4]])
    np.testing.assert_array_equal((2.0 * x).evaluate_global(pts), (2.0 * x).evaluate(pts))
    assert (x[0] + 1.0).evaluate_global(0.5).tolist() == [[1.5]]
    mesh = uw.mesh.FeMesh_Cartesian(elementRes=(2, 2))
    with pytest.raises(TypeError, match="not currently supported"):
        x.evaluate_global(mesh)
    with pytest.raises(TypeError, match="not currently supported"):
        x.evaluate_global(mesh.specialSets["MinI_VertexSet"])


def test_mesh_variable_outside_the_mesh():
    """FeVariableFn.cpp:82-92: a mesh variable evaluated at a coordinate outside
    its mesh raises ValueError naming the location (checked before any
    interpolation, so this runs without a GPU)."""
    mesh = uw.mesh.FeMesh_Cartesian(elementRes=(4, 4))
    var = uw.mesh.MeshVariable(mesh, 1)
    with pytest.raises(ValueError, match=r"location \(2, 0.5\) does not appear to be valid"):
        var.evaluate((2.0, 0.5))
    with pytest.raises(ValueError, match="outside local domain"):
        (2.0 * var.fn_gradient[0]).evaluate(np.array([[0.5, 0.5], [0.5, -0.1]]))
    with pytest.raises(RuntimeError, match="No results were found"):
        var.evaluate_global(np.array([[1.5, 0.5], [-0.5, 0.5]]))
