"""Known answers from the reference's IndexSet docstrings
(P/container/_indexset.py:20-604, P/mesh/_mesh.py:1228-1266), restated as
tests (CPU): construction, add / remove / AND, membership, data, length,
invert / addAll / clear and the set operators, with the reference's reprs."""
import numpy as np
import pytest

import underworld2_gb300 as uw
from underworld2_gb300.container import IndexSet


def test_construction_and_add():
    s = IndexSet(15, [3, 14, 2])
    assert repr(s) == "IndexSet([ 2,  3, 14])"
    s = IndexSet(15)
    assert repr(s) == "IndexSet([])"
    s.add(3)
    assert repr(s) == "IndexSet([3])" and 3 in s
    s.add([2, 11])
    assert repr(s) == "IndexSet([ 2,  3, 11])"
    s = IndexSet(15)
    s.add(3)
    s.add([5, 3, 7, 8])
    assert repr(s) == "IndexSet([3, 5, 7, 8])"
    s.add(np.array([10, 11, 3]))
    assert repr(s) == "IndexSet([ 3,  5,  7,  8, 10, 11])"


def test_remove_and_membership():
    s = IndexSet(15, [3, 9, 10])
    assert repr(s) == "IndexSet([ 3,  9, 10])" and 3 in s
    s.remove(3)
    assert 3 not in s and repr(s) == "IndexSet([ 9, 10])"
    s.remove([9, 10])
    assert repr(s) == "IndexSet([])"


def test_data_length_and_in_place_edits():
    s = IndexSet(15, [3, 9, 10])
    assert s.data.dtype == np.uint32 and s.data.tolist() == [3, 9, 10] and not s.data.flags.writeable
    assert len(s) == 3
    s = IndexSet(15, [1, 3, 5, 7, 9, 11, 13])
    s.invert()
    assert repr(s) == "IndexSet([ 0,  2,  4,  6,  8, 10, 12, 14])"
    s = IndexSet(5)
    s.addAll()
    assert repr(s) == "IndexSet([0, 1, 2, 3, 4])"
    s = IndexSet(5, [1, 2, 3])
    s.clear()
    assert repr(s) == "IndexSet([])"


def test_operators():
    a, b = IndexSet(15, [3, 9, 10]), IndexSet(15, [1, 9, 12])
    assert repr(a + b) == "IndexSet([ 1,  3,  9, 10, 12])"
    assert repr(a - b) == "IndexSet([ 3, 10])"
    assert repr(a & b) == "IndexSet([9])"
    assert repr(a | b) == "IndexSet([ 1,  3,  9, 10, 12])"
    for op, expect in (("__iadd__", "IndexSet([ 1,  3,  9, 10, 12])"), ("__isub__", "IndexSet([ 3, 10])"),
                       ("__iand__", "IndexSet([9])")):
        c = IndexSet(15, [3, 9, 10])
        getattr(c, op)(b)
        assert repr(c) == expect
    a.AND(b)
    assert repr(a) == "IndexSet([9])"


def test_argument_checks():
    with pytest.raises(ValueError):
        IndexSet(0)
    with pytest.raises(ValueError):
        IndexSet(15, [15])
    with pytest.raises(ValueError):
        IndexSet(15).add(-1)
    with pytest.raises(TypeError):
        IndexSet(15) + [1, 2]
    with pytest.raises(ValueError):
        IndexSet(15) + IndexSet(16)


def test_mesh_vertex_sets():
    """FeMesh_IndexSet docstring: the MaxI vertices of a 4 x 4 Q1 mesh; special sets
    are new objects on every lookup; functions evaluate on a vertex set."""
    m = uw.mesh.FeMesh_Cartesian(elementType="Q1/dQ0", elementRes=(4, 4), minCoord=(0.0, 0.0), maxCoord=(1.0, 1.0))
    s = m.specialSets["MaxI_VertexSet"]
    assert repr(s) == "FeMesh_IndexSet([ 4,  9, 14, 19, 24])" and s.topologicalIndex == 0 and s.object is m
    iset = uw.mesh.FeMesh_IndexSet(m, topologicalIndex=0, size=m.nodesGlobal, fromObject=s.data)
    assert repr(iset) == "FeMesh_IndexSet([ 4,  9, 14, 19, 24])"
    e = m.specialSets["Empty"]
    e.add(3)
    assert len(m.specialSets["Empty"]) == 0
    left = m.specialSets["Left_VertexSet"]
    hand = m.specialSets["Empty"]
    for index, coord in enumerate(m.data):
        if coord[0] < 0.01:
            hand.add(index)
    assert len(left) == len(hand) and np.allclose(left, hand)
    full = m.specialSets["Empty"]
    full.invert()
    fn_k = 5.0 + 8.0 * uw.function.math.exp(5.0 * uw.function.input()[1])
    np.testing.assert_array_equal(fn_k.evaluate(full), fn_k.evaluate(m.data))
