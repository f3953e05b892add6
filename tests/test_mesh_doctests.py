"""Known answers from the reference's FeMesh docstrings (P/mesh/_mesh.py:185-560),
restated as tests (CPU): vertex array shape and values, global / local /
domain sizes, the special sets' names and members, and a save / load round
trip onto a mesh of another extent.  (The deform_mesh examples are outside
this package, whose meshes stay regular.)"""
import numpy as np

import underworld2_gb300 as uw


def test_sizes_and_vertices():
    m = uw.mesh.FeMesh_Cartesian(elementType="Q1", elementRes=(2, 2), minCoord=(-1.0, -1.0), maxCoord=(1.0, 1.0))
    assert m.data.shape == (9, 2)
    np.testing.assert_array_equal(m.data[1], [0.0, -1.0])
    assert m.nodesGlobal == 9
    assert m.elementsLocal == 4 and m.elementsDomain == 4 and m.elementsGlobal == 4


def test_special_sets():
    m = uw.mesh.FeMesh_Cartesian(elementType="Q1", elementRes=(2, 2), minCoord=(0.0, 0.0), maxCoord=(1.0, 1.0))
    assert sorted(m.specialSets.keys()) == ["AllWalls_VertexSet", "Bottom_VertexSet", "Empty", "Left_VertexSet",
                                            "MaxI_VertexSet", "MaxJ_VertexSet", "MinI_VertexSet", "MinJ_VertexSet",
                                            "Right_VertexSet", "Top_VertexSet"]
    assert repr(m.specialSets["MinJ_VertexSet"]) == "FeMesh_IndexSet([0, 1, 2])"


def test_save_and_load_onto_another_extent(tmp_path):
    mesh = uw.mesh.FeMesh_Cartesian(elementType="Q1/dQ0", elementRes=(16, 16), minCoord=(0.0, 0.0), maxCoord=(1.0, 1.0))
    mesh.save(str(tmp_path / "saved_mesh.h5"))
    clone = uw.mesh.FeMesh_Cartesian(elementType="Q1/dQ0", elementRes=(16, 16), minCoord=(0.0, 0.0),
                                     maxCoord=(1.5, 1.5))
    assert not np.allclose(mesh.data, clone.data)
    clone.load(str(tmp_path / "saved_mesh.h5"))
    assert np.allclose(mesh.data, clone.data)
