"""Checkpoint files: the HDF5 subset writer/reader, mesh and variable
save/load, XDMF descriptions (P/mesh/_mesh.py:495-675,
P/mesh/_meshvariable.py:227-620, P/swarm/_swarm.py:226-420,
P/swarm/_swarmvariable.py:244-600 and their docstring examples)."""
import os
import struct
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from oracle.ref_analytic import REFERENCE_TREE
from underworld2_gb300 import h5


def _roundtrip(tmp_path, datasets, attrs):
    fn = str(tmp_path / "t.h5")
    h5.write(fn, datasets, attrs)
    return fn, h5.File(fn)


def test_h5_roundtrip_datasets_and_attributes(tmp_path):
    rng = np.random.default_rng(0)
    ds = {"vertices": rng.standard_normal((17, 3)), "en_map": rng.integers(0, 99, (5, 8)).astype(np.int32),
          "w": rng.standard_normal(11).astype(np.float32), "empty": np.zeros((0, 3)),
          "big": np.arange(6, dtype=np.int64).reshape(2, 3), "flags": np.array([1, 0, 1], dtype=np.uint8)}
    at = {"dimensions": 3, "mesh resolution": (4, 5, 6), "max": (1.0, 2.0, 3.5), "min": (0.0, -1.0, 0.5),
          "regular": True, "elementType": "Q2", "raw": np.bytes_(b"DPC1"), "proc_offset": np.array([17]),
          "pi": 3.25}
    fn, f = _roundtrip(tmp_path, ds, at)
    assert sorted(f.keys()) == sorted(ds)
    for k, v in ds.items():
        r = f[k]
        assert r.dtype == v.dtype and r.shape == v.shape
        np.testing.assert_array_equal(r, v)
    assert f.attrs["dimensions"] == 3
    assert tuple(f.attrs["mesh resolution"]) == (4, 5, 6)
    np.testing.assert_array_equal(f.attrs["max"], [1.0, 2.0, 3.5])
    assert bool(f.attrs["regular"]) is True
    assert f.attrs["elementType"] == b"Q2"
    assert f.attrs["raw"] == b"DPC1"
    assert list(f.attrs["proc_offset"]) == [17]
    assert f.attrs["pi"] == 3.25


def test_h5_file_structure(tmp_path):
    """Invariants of the format as written: signature, end-of-file address,
    superblock root entry matching the root symbol-table message, signatures of
    the B-tree, symbol table node and local heap, 8-byte aligned headers and
    message sizes, raw data inside the file."""
    fn, f = _roundtrip(tmp_path, {"a": np.arange(10.0), "b": np.ones((3, 2), np.int32)}, {"x": 1})
    b = open(fn, "rb").read()
    assert b[:8] == b"\x89HDF\r\n\x1a\n"
    assert b[8] == 0 and b[13] == 8 and b[14] == 8
    leaf_k, int_k = struct.unpack_from("<HH", b, 16)
    eof = struct.unpack_from("<Q", b, 40)[0]
    assert eof == len(b)
    root, cache = struct.unpack_from("<QI", b, 64)
    bt, hp = struct.unpack_from("<QQ", b, 80)
    assert cache == 1 and root % 8 == 0
    assert b[root] == 1
    nmsg, _, size = struct.unpack_from("<HII", b, root + 2)
    p = root + 16
    found = False
    for _ in range(nmsg):
        mtype, msize = struct.unpack_from("<HH", b, p)
        assert msize % 8 == 0
        if mtype == 0x0011:
            assert struct.unpack_from("<QQ", b, p + 8) == (bt, hp)
            found = True
        p += 8 + msize
    assert found and p == root + 16 + size
    assert b[bt:bt + 4] == b"TREE"
    snod = struct.unpack_from("<Q", b, bt + 32)[0]
    assert b[snod:snod + 4] == b"SNOD" and struct.unpack_from("<H", b, snod + 6)[0] == 2
    assert b[hp:hp + 4] == b"HEAP"
    dsize, free, daddr = struct.unpack_from("<QQQ", b, hp + 8)
    assert free == 1 and daddr + dsize <= len(b) and b[daddr] == 0
    for k in range(2):
        oh = struct.unpack_from("<Q", b, snod + 8 + 40 * k + 8)[0]
        assert oh % 8 == 0 and b[oh] == 1


def test_h5_rejects_non_hdf5(tmp_path):
    fn = tmp_path / "x.h5"
    fn.write_bytes(b"not an hdf5 file at all")
    with pytest.raises(ValueError):
        h5.File(str(fn))


def test_element_node_map():
    import underworld2_gb300 as uw
    for et, res in [("Q1/dQ0", (3, 2)), ("Q2/dPc1", (2, 3)), ("Q1/dQ0", (2, 2, 3)), ("Q2/dPc1", (2, 1, 2))]:
        m = uw.mesh.FeMesh_Cartesian(et, res, (0.0,) * len(res), (1.0,) * len(res))
        en = m.data_elementNodes
        o = m._order
        n = [r * o + 1 for r in res]
        for e in range(m.elementsGlobal):
            ei = [e % res[0], (e // res[0]) % res[1]] + ([e // (res[0] * res[1])] if len(res) == 3 else [])
            k = 0
            for c in range(o + 1 if len(res) == 3 else 1):
                for b in range(o + 1):
                    for a in range(o + 1):
                        g = (ei[0] * o + a) + n[0] * (ei[1] * o + b)
                        if len(res) == 3:
                            g += n[0] * n[1] * (ei[2] * o + c)
                        assert en[e, k] == g
                        k += 1
        # every element's nodes enclose its centroid
        x = m.data[en]
        lo, hi = x.min(1), x.max(1)
        assert np.all(hi - lo > 0)


def test_mesh_and_variable_save_load(tmp_path):
    """The reference's docstring example: save a 16x16 mesh and a variable,
    reload the mesh into a clone with another extent and the variable into a
    clone variable."""
    import underworld2_gb300 as uw
    mesh = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (16, 16), (0.0, 0.0), (1.0, 1.0))
    var = uw.mesh.MeshVariable(mesh=mesh, nodeDofCount=1, dataType="double")
    var.data[:, 0] = np.arange(var.data.shape[0])
    mh = mesh.save(str(tmp_path / "saved_mesh.h5"))
    assert isinstance(mh, uw.utils.SavedFileData) and os.path.isabs(mh.filename)
    var.save(str(tmp_path / "saved_mesh_variable.h5"), mh)
    var.save(str(tmp_path / "saved_mesh_variable.h5"), mh)   # overwrite
    clone = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (16, 16), (0.0, 0.0), (1.5, 1.5))
    assert not np.allclose(mesh.data, clone.data)
    clone.load(str(tmp_path / "saved_mesh.h5"))
    assert np.allclose(mesh.data, clone.data)
    cv = uw.mesh.MeshVariable(mesh=mesh, nodeDofCount=1, dataType="double")
    cv.load(str(tmp_path / "saved_mesh_variable.h5"))
    assert np.allclose(var.data, cv.data)
    f = h5.File(str(tmp_path / "saved_mesh.h5"))
    assert tuple(f.attrs["mesh resolution"]) == (16, 16) and f.attrs["dimensions"] == 2
    assert f["en_map"].shape == (256, 4) and f["vertices"].shape == (289, 2)
    g = h5.File(str(tmp_path / "saved_mesh_variable.h5"))
    assert g.attrs["mesh"] == mh.filename.encode()
    # a different resolution needs interpolate=True
    m19 = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (19, 19), (0.0, 0.0), (1.0, 1.0))
    v19 = m19.add_variable(1)
    with pytest.raises(RuntimeError):
        v19.load(str(tmp_path / "saved_mesh_variable.h5"))
    # pressure (sub-mesh) variables
    pv = mesh.subMesh.add_variable(1)
    pv.data[:, 0] = np.linspace(0, 1, pv.data.shape[0])
    pv.save(str(tmp_path / "p.h5"), mh)
    pv2 = mesh.subMesh.add_variable(1)
    pv2.load(str(tmp_path / "p.h5"))
    np.testing.assert_array_equal(pv.data, pv2.data)
    assert h5.File(str(tmp_path / "p.h5")).attrs["elementType"] == b"DQ0"


def test_mesh_load_rejects_deformed(tmp_path):
    import underworld2_gb300 as uw
    from underworld2_gb300 import h5 as H
    mesh = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (4, 4), (0.0, 0.0), (1.0, 1.0))
    v = mesh.data.copy()
    v[7, 0] += 0.01
    H.write(str(tmp_path / "d.h5"), {"vertices": v, "en_map": mesh.data_elementNodes}, {"regular": False})
    with pytest.raises(NotImplementedError):
        mesh.load(str(tmp_path / "d.h5"))


@pytest.mark.parametrize("et,res,dof", [("Q1/dQ0", (4, 3), 1), ("Q1/dQ0", (4, 3), 2), ("Q2/dPc1", (2, 2, 2), 3),
                                        ("Q1/dQ0", (2, 2, 2), 6), ("Q1/dQ0", (3, 3), 4)])
def test_mesh_variable_xdmf(tmp_path, et, res, dof):
    import underworld2_gb300 as uw
    mesh = uw.mesh.FeMesh_Cartesian(et, res, (0.0,) * len(res), (1.0,) * len(res))
    var = mesh.add_variable(dof)
    mh = mesh.save(str(tmp_path / "m.h5"))
    vh = var.save(str(tmp_path / "v.h5"), mh)
    var.xdmf(str(tmp_path / "out"), vh, "field", mh, "mesh", modeltime=1.5)
    root = ET.parse(str(tmp_path / "out.xdmf")).getroot()
    grid = root.find("Domain/Grid")
    assert grid.find("Time").get("Value") == "1.5"
    topo = grid.find("Topology")
    assert int(topo.get("NumberOfElements")) == mesh.elementsGlobal
    join = topo.find("DataItem")
    nen = (mesh._order + 1) ** mesh.dim
    assert join.get("Dimensions") == "%d %d" % (mesh.elementsGlobal, nen)
    cols = sorted(int(t.strip().lstrip("$")) for t in join.get("Function")[5:-1].split(","))
    assert cols == list(range(nen))
    refs = [d.text for d in root.iter("DataItem") if d.get("Format") == "HDF"]
    assert any(r.endswith("m.h5:/en_map") for r in refs) and any(r.endswith("m.h5:/vertices") for r in refs)
    assert any(r.endswith("v.h5:/data") for r in refs)
    with pytest.raises(RuntimeError):
        other = uw.mesh.FeMesh_Cartesian(et, res, (0.0,) * len(res), (1.0,) * len(res))
        var.xdmf(str(tmp_path / "bad"), vh, "field", other.save(str(tmp_path / "o.h5")), "mesh")


@pytest.mark.gpu
def test_swarm_and_variable_save_load(tmp_path):
    """Swarm + swarm variable round trip through the checkpoint files, a
    swarm loaded into a fresh swarm keeps the saved order and values, and an
    interpolated mesh-variable load of a linear field is exact."""
    import underworld2_gb300 as uw
    mesh = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (8, 8), (0.0, 0.0), (1.0, 1.0))
    sw = uw.swarm.Swarm(mesh)
    sw.populate_using_layout(uw.swarm.layouts.PerCellRandomLayout(sw, 5, seed=13))
    mat = sw.add_variable("int", 1)
    mat.data[:, 0] = np.arange(sw.particleLocalCount) % 7
    temp = sw.add_variable("double", 2)
    temp.data[:] = sw.data * 2.0
    sh = sw.save(str(tmp_path / "swarm.h5"))
    mh = mat.save(str(tmp_path / "mat.h5"), swarmHandle=sh)
    th = temp.save(str(tmp_path / "temp.h5"), sh)
    sw2 = uw.swarm.Swarm(mesh)
    mat2 = sw2.add_variable("int", 1)
    temp2 = sw2.add_variable("double", 2)
    sw2.load(str(tmp_path / "swarm.h5"))
    mat2.load(str(tmp_path / "mat.h5"))
    temp2.load(str(tmp_path / "temp.h5"))
    np.testing.assert_array_equal(sw2.data, sw.data)
    np.testing.assert_array_equal(mat2.data, mat.data)
    np.testing.assert_array_equal(temp2.data, temp.data)
    mat.xdmf(str(tmp_path / "mat"), mh, "material", sh, "swarm")
    root = ET.parse(str(tmp_path / "mat.xdmf")).getroot()
    assert root.find("Domain/Grid/Topology").get("NodesPerElement") == str(sw.particleLocalCount)
    # loading a variable before its swarm is refused
    sw3 = uw.swarm.Swarm(mesh)
    v3 = sw3.add_variable("double", 2)
    with pytest.raises(RuntimeError):
        v3.load(str(tmp_path / "temp.h5"))
    # interpolated mesh-variable load (linear data: exact on Q1)
    var = mesh.add_variable(1)
    var.data[:, 0] = 1.0 + 2.0 * mesh.data[:, 0] - 0.5 * mesh.data[:, 1]
    vmh = mesh.save(str(tmp_path / "m.h5"))
    var.save(str(tmp_path / "v.h5"), vmh)
    m19 = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (19, 19), (0.0, 0.0), (1.0, 1.0))
    v19 = m19.add_variable(1)
    v19.load(str(tmp_path / "v.h5"), interpolate=True)
    np.testing.assert_allclose(v19.data[:, 0], 1.0 + 2.0 * m19.data[:, 0] - 0.5 * m19.data[:, 1], atol=1e-12)


def _pad8(b):
    return b + b"\0" * ((-len(b)) % 8)


def test_h5_reader_continuation_and_vlen_strings():
    """Reader paths that libhdf5-written files use: an object header whose
    messages continue in a second block (continuation message 0x0010), and a
    variable-length string attribute whose bytes live in a global heap
    collection (how h5py stores Python str attributes).  Byte layouts follow
    the HDF5 file-format specification."""
    import struct
    from underworld2_gb300.h5 import _Reader
    # global heap collection at 256: object 1 = b"Q2"
    text = b"Q2"
    obj = struct.pack("<HH4xQ", 1, 1, len(text)) + _pad8(text)
    gcol = b"GCOL" + bytes([1, 0, 0, 0]) + struct.pack("<Q", 16 + len(obj) + 16) + obj + b"\0" * 16
    # attribute "elementType": class 9 (variable length), type 1 (string), size 16,
    # base type: 1-byte string; scalar dataspace; value = (length, heap address, index)
    base = bytes([0x10 | 3, 0, 0, 0]) + struct.pack("<I", 1)
    dt = bytes([0x10 | 9, 0x01, 0, 0]) + struct.pack("<I", 16) + base
    sp = bytes([1, 0, 0, 0]) + b"\0" * 4
    name = b"elementType\0"
    body = struct.pack("<BxHHH", 1, len(name), len(dt), len(sp)) + _pad8(name) + _pad8(dt) + _pad8(sp) + \
        struct.pack("<IQI", len(text), 256, 1)
    body = _pad8(body)
    amsg = struct.pack("<HHB3x", 0x000C, len(body), 0) + body
    # object header at 0: one continuation message pointing at the block at 64
    cont = struct.pack("<HHB3x", 0x0010, 16, 0) + struct.pack("<QQ", 64, len(amsg))
    hdr = struct.pack("<BxHII4x", 1, 2, 1, len(cont)) + cont
    buf = bytearray(512)
    buf[0:len(hdr)] = hdr
    buf[64:64 + len(amsg)] = amsg
    buf[256:256 + len(gcol)] = gcol
    r = _Reader(bytes(buf))
    msgs = r.messages(0)
    assert [m[0] for m in msgs] == [0x0010, 0x000C]
    name_out, value = r.attribute(msgs[1][1])
    assert name_out == "elementType" and value == "Q2"


_REF_INPUT = os.path.join(REFERENCE_TREE, "docs", "examples", "input")


@pytest.mark.skipif(not os.path.isdir(_REF_INPUT), reason="reference tree not present")
def test_h5_reader_on_reference_swarm_files():
    """The swarm checkpoints the reference ships with its shear-band example,
    written by h5py/libhdf5 (docs/examples/input/07_ShearBandsPureShear): 28,800
    particle coordinates in the example's [-2, 2] x [0, 1] box and their plastic
    strain, each with the proc_offset attribute of a one-process save."""
    d = os.path.join(_REF_INPUT, "07_ShearBandsPureShear")
    f = h5.File(os.path.join(d, "particle_coords.h5"))
    x = f["data"]
    assert x.shape == (28800, 2) and x.dtype == np.float64
    assert x[:, 0].min() > -2.0 and x[:, 0].max() < 2.0 and x[:, 1].min() > 0.0 and x[:, 1].max() < 1.0
    assert f.attrs["proc_offset"].tolist() == [28800] and f.links == {}
    g = h5.File(os.path.join(d, "plastic_strain.h5"))
    e = g["data"]
    assert e.shape == (28800, 1) and e.min() >= 0.0 and e.max() < 1.0
    assert g.attrs["proc_offset"].tolist() == [28800]
