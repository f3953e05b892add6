"""Known answers from the reference's MeshVariable docstrings
(P/mesh/_meshvariable.py:48-160, 258-400, 630-644), restated as tests (CPU):
data layout, the checkpoint round trip with its XDMF file, and copy.  (The
interpolating load and the evaluate examples need the GPU and are covered by
the GPU tests.)"""
import math
import os

import numpy as np

import underworld2_gb300 as uw


def test_data_layout():
    linearMesh = uw.mesh.FeMesh_Cartesian(elementType="Q1/dQ0", elementRes=(16, 16), minCoord=(0.0, 0.0),
                                          maxCoord=(1.0, 1.0))
    scalarFeVar = uw.mesh.MeshVariable(mesh=linearMesh, nodeDofCount=1, dataType="double")
    assert scalarFeVar.data.shape == (289, 1)
    assert scalarFeVar.data[100].tolist() == [0.0]
    scalarFeVar.data[100] = 15.333
    assert scalarFeVar.data[100].tolist() == [15.333]
    vectorFeVar = uw.mesh.MeshVariable(mesh=linearMesh, nodeDofCount=3, dataType="double")
    assert vectorFeVar.data.shape == (289, 3)


def test_save_xdmf_and_load(tmp_path):
    mesh = uw.mesh.FeMesh_Cartesian(elementType="Q1/dQ0", elementRes=(16, 16), minCoord=(0.0, 0.0), maxCoord=(1.0, 1.0))
    var = uw.mesh.MeshVariable(mesh=mesh, nodeDofCount=1, dataType="double")
    var.data[:, 0] = np.arange(var.data.shape[0])
    meshDat = mesh.save(str(tmp_path / "saved_mesh.h5"))
    varDat = var.save(str(tmp_path / "saved_mesh_variable.h5"), meshDat)
    var.save(str(tmp_path / "saved_mesh_variable.h5"), meshDat)          # saving again overwrites
    var.xdmf(str(tmp_path / "TESTxdmf"), varDat, "var1", meshDat, "meshie")
    assert os.path.isfile(str(tmp_path / "TESTxdmf.xdmf"))
    clone_var = uw.mesh.MeshVariable(mesh=mesh, nodeDofCount=1, dataType="double")
    clone_var.load(str(tmp_path / "saved_mesh_variable.h5"))
    assert np.allclose(var.data, clone_var.data)


def test_copy():
    mesh = uw.mesh.FeMesh_Cartesian()
    var = uw.mesh.MeshVariable(mesh, 2)
    var.data[:] = (math.pi, math.exp(1.0))
    varCopy = var.copy()
    assert varCopy.mesh == var.mesh and varCopy.nodeDofCount == var.nodeDofCount
    assert not np.allclose(var.data, varCopy.data)
    varCopy2 = var.copy(deepcopy=True)
    assert np.allclose(var.data, varCopy2.data)
