"""Regular Cartesian FE meshes and mesh variables (``uw.mesh`` subset).

Mirrors ``FeMesh_Cartesian`` / ``MeshVariable`` of the reference
(P/mesh/_mesh.py:1105-1160, P/mesh/_meshvariable.py) for Q1/dQ0 meshes:
node numbering x-fastest, element numbering x-fastest, node coordinates
``min + (i/n)*(max-min)`` (L/StgDomain/Mesh/src/CartesianGenerator.c:2003-2036).
``MeshVariable.data`` is a host numpy array; the library copies it to the
device when a solve or an advection reads it and writes results back in place.
"""
import copy
import os
import re

import numpy as np
import torch

from . import _core
from . import function as _fn
from . import h5 as _h5
from . import utils as _utils
from . import container as _container
from .container import ObjectifiedIndexSet


class FeMesh_IndexSet(ObjectifiedIndexSet):
    """Indices of a mesh's vertices (topologicalIndex 0), edges, faces or volumes,
    tied to the mesh (P/mesh/_mesh.py:1228-1266); functions evaluate on it at
    those vertices."""

    def __init__(self, object, topologicalIndex=None, *args, **kwargs):
        if topologicalIndex not in (0, 1, 2, 3):
            raise ValueError("Topological index must be within [0,3].")
        if not isinstance(object, FeMesh_Cartesian):
            raise TypeError("'object' parameter must be of (sub)type 'FeMesh'.")
        self._toplogicalIndex = topologicalIndex
        super().__init__(object, *args, **kwargs)

    @property
    def topologicalIndex(self):
        """0 vertex, 1 edge, 2 face, 3 volume."""
        return self._toplogicalIndex


IndexSet = _container.IndexSet     # the plain container, kept under its earlier name here


class FeMesh_Cartesian:
    """Regular Cartesian mesh: ``elementType`` 'Q1/dQ0' or 'Q2/dPc1' (2D and 3D):
    primary velocity mesh and the pressure sub-mesh."""

    def __init__(self, elementType="Q1/dQ0", elementRes=(4, 4), minCoord=(0.0, 0.0), maxCoord=(1.0, 1.0),
                 periodic=None, partitioned=True, **kwargs):
        if isinstance(elementType, str):
            elementType = re.split(",|-|/", elementType)
        types = [t.upper() for t in elementType]
        if types[0] == "Q1" and (len(types) == 1 or types[1] == "DQ0"):
            order, porder = 1, 0
        elif types[0] == "Q2" and (len(types) == 1 or types[1] == "DPC1"):
            order, porder = 2, 1
        else:
            raise ValueError("supported element types: 'Q1/dQ0' and 'Q2/dPc1' (got %s)" % "/".join(elementType))
        if periodic and any(periodic):
            raise ValueError("periodic meshes are not supported")
        if len(elementRes) not in (2, 3) or len(minCoord) != len(elementRes) or len(maxCoord) != len(elementRes):
            raise ValueError("elementRes, minCoord and maxCoord must have the same length (2 or 3)")
        self.dim = len(elementRes)
        self.elementRes = tuple(int(r) for r in elementRes)
        self.minCoord = tuple(float(v) for v in minCoord)
        self.maxCoord = tuple(float(v) for v in maxCoord)
        self.elementType = "Q%d" % order
        self._order, self._porder = order, porder
        self._ctx = None
        n = [r * order + 1 for r in self.elementRes]
        self.nodesGlobal = int(np.prod(n))
        self.elementsGlobal = int(np.prod(self.elementRes))
        self._axes = [self.minCoord[d] + (np.arange(n[d]) / (n[d] - 1)) * (self.maxCoord[d] - self.minCoord[d])
                      for d in range(self.dim)]
        for d in range(self.dim):
            self._axes[d][0], self._axes[d][-1] = self.minCoord[d], self.maxCoord[d]
        self.subMesh = _SubMesh(self)
        self.specialSets = _SpecialSets(self)

    @property
    def ctx(self):
        if self._ctx is None:
            self._ctx = _core.Context(self.dim, self.elementRes, self.minCoord, self.maxCoord,
                                      order=self._order, porder=self._porder)
        return self._ctx

    @property
    def data(self):
        """Node coordinates [nodes, dim], node index x-fastest."""
        g = np.meshgrid(*self._axes, indexing="ij")
        return np.stack([a.transpose().ravel() for a in g], axis=1)

    @property
    def nodesLocal(self):
        return self.nodesGlobal

    @property
    def elementsLocal(self):
        return self.elementsGlobal

    @property
    def nodesDomain(self):
        """Local plus shadow nodes (P/mesh/_mesh.py:373-380); one process holds them all."""
        return self.nodesGlobal

    @property
    def elementsDomain(self):
        """Local plus shadow elements (P/mesh/_mesh.py:391-405)."""
        return self.elementsGlobal

    def add_variable(self, nodeDofCount, dataType="double", **kwargs):
        return MeshVariable(self, nodeDofCount, dataType)

    @property
    def data_elementNodes(self):
        """Element-node map [elements, nodes per element]: global node indices,
        element x-fastest, nodes of an element in lexicographic order."""
        o, r, dim = self._order, self.elementRes, self.dim
        n = [ri * o + 1 for ri in r]
        k = o + 1
        e = np.arange(self.elementsGlobal)
        ei = [e % r[0], (e // r[0]) % r[1]] + ([e // (r[0] * r[1])] if dim == 3 else [])
        loc = np.arange(k ** dim)
        li = [loc % k, (loc // k) % k] + ([loc // (k * k)] if dim == 3 else [])
        g = [ei[d][:, None] * o + li[d][None, :] for d in range(dim)]
        node = g[0] + n[0] * g[1]
        if dim == 3:
            node = node + n[0] * n[1] * g[2]
        return node.astype(np.int32)

    # -- checkpointing (P/mesh/_mesh.py:495-675) -----------------------------
    def save(self, filename, units=None, **kwargs):
        """Write the mesh to an HDF5 file: ``vertices`` [nodes, dim], ``en_map``
        [elements, nodes per element] and the attributes dimensions, mesh
        resolution, max, min, regular and elementType (plus ``kwargs`` as
        strings).  Returns a ``SavedFileData``."""
        if not isinstance(filename, str):
            raise TypeError("Expected 'filename' to be provided as a string")
        if units is not None:
            raise NotImplementedError("saving with units (dimensional scaling) is not supported")
        attrs = {"dimensions": self.dim, "mesh resolution": self.elementRes, "max": self.maxCoord,
                 "min": self.minCoord, "regular": True, "elementType": self.elementType}
        attrs.update({str(k): str(v) for k, v in kwargs.items()})
        _h5.write(filename, {"vertices": self.data, "en_map": self.data_elementNodes}, attrs)
        return _utils.SavedFileData(self, filename)

    def load(self, filename):
        """Read mesh vertices saved by ``save``.  The mesh stays regular: the
        vertices must form the regular grid of this resolution, whose extent
        becomes the mesh's ``minCoord``/``maxCoord``."""
        if not isinstance(filename, str):
            raise TypeError("Expected 'filename' to be provided as a string")
        with _h5.File(filename) as f:
            v = f["vertices"]
        if v.shape[1] != self.dim:
            raise RuntimeError("Can't load hdf5 '%s', incompatible data shape" % filename)
        if v.shape[0] != self.nodesGlobal:
            raise RuntimeError("Provided data file appears to be for a different resolution mesh.")
        (ii, nn) = self._node_grid()
        axes = []
        for d in range(self.dim):
            ax = np.zeros(nn[d])
            ax[ii[d]] = v[:, d]
            if not np.array_equal(ax[ii[d]], v[:, d]) or np.any(np.diff(ax) <= 0):
                raise NotImplementedError("the saved mesh is deformed; only regular meshes are supported")
            axes.append(ax)
        lo = tuple(float(a[0]) for a in axes)
        hi = tuple(float(a[-1]) for a in axes)
        mesh = FeMesh_Cartesian("Q%d/%s" % (self._order, "dQ0" if self._porder == 0 else "dPc1"),
                                self.elementRes, lo, hi)
        if any(not np.allclose(mesh._axes[d], axes[d], rtol=0, atol=1e-12 * (1 + abs(hi[d] - lo[d])))
               for d in range(self.dim)):
            raise NotImplementedError("the saved mesh is deformed; only regular meshes are supported")
        self.minCoord, self.maxCoord = lo, hi
        self._axes = mesh._axes
        self._ctx = None

    def integrate(self, fn):
        """Volume integral of fn over the mesh (P/mesh/_mesh.py:1200-1226)."""
        from .utils import Integral
        return Integral(fn, mesh=self).evaluate()

    def _node_grid(self):
        n = [r * self._order + 1 for r in self.elementRes]
        idx = np.arange(self.nodesGlobal)
        out = [idx % n[0], (idx // n[0]) % n[1]]
        if self.dim == 3:
            out.append(idx // (n[0] * n[1]))
        return out, n


# Faces of an element in the reference's border-layout numbering
# (GaussBorderParticleLayout.c:300-320): faces 0, 1 lie at y = -1, +1, faces 2, 3
# at x = -1, +1, faces 4, 5 at z = -1, +1 (even faces at -1, odd at +1).
_FACE_AXIS = (1, 1, 0, 0, 2, 2)


def _border_points(mesh, node_on, n_gauss):
    """Gauss points on the faces of the elements that hold a flagged node
    (GaussBorderParticleLayout.c:186-290), kept where the interpolated node
    indicator exceeds 0.999 (the mask of P/systems/sle/_assemblyterm.py:124-144
    and P/utils/_utils.py:131-142).  Returns numpy arrays: global coordinates
    [q, dim], weight x surface Jacobian [q] (ElementType.c:566-606: the product
    of h_j / 2 over the face's axes), shape values [q, nen] and element nodes
    [q, nen] of the kept points."""
    dim, o = mesh.dim, mesh._order
    en = mesh.data_elementNodes.astype(np.int64)
    flagged = np.nonzero(node_on[en].any(1))[0]
    x1, w1 = np.polynomial.legendre.leggauss(n_gauss)
    pts, wts, fax = [], [], []
    for f in range(2 * dim):
        k = _FACE_AXIS[f]
        others = [a for a in range(dim) if a != k]
        for idx in np.ndindex(*([n_gauss] * (dim - 1))):
            xi = np.zeros(dim)
            xi[k] = -1.0 if f % 2 == 0 else 1.0
            w = 1.0
            for a, i in zip(others, idx):
                xi[a] = x1[i]
                w *= w1[i]
            pts.append(xi)
            wts.append(w)
            fax.append(k)
    pts, wts, fax = np.array(pts), np.array(wts), np.array(fax)
    kk = o + 1
    loc = np.arange(kk ** dim)
    li = [loc % kk, (loc // kk) % kk] + ([loc // (kk * kk)] if dim == 3 else [])
    N = np.ones((len(pts), kk ** dim))
    for d in range(dim):
        s_ = pts[:, d]
        b = np.stack([(1 - s_) / 2, (1 + s_) / 2], 1) if o == 1 else \
            np.stack([0.5 * s_ * (s_ - 1), 1 - s_ * s_, 0.5 * s_ * (s_ + 1)], 1)
        N *= b[:, li[d]]
    r = mesh.elementRes
    ei = [flagged % r[0], (flagged // r[0]) % r[1]] + ([flagged // (r[0] * r[1])] if dim == 3 else [])
    det = np.ones((len(flagged), len(pts)))
    for d in range(dim):
        h = mesh._axes[d][(ei[d] + 1) * o] - mesh._axes[d][ei[d] * o]
        det *= np.where(fax[None, :] == d, 1.0, (h / 2.0)[:, None])
    enf = en[flagged]
    delta = node_on.astype(np.float64)[enf] @ N.T
    fe, pe = np.nonzero(delta > 0.999)
    xg = np.einsum("qa,qad->qd", N[pe], mesh.data[enf[fe]])
    return xg, wts[pe] * det[fe, pe], N[pe], enf[fe]


def _volume_points(mesh, n_gauss, first, count):
    """Global coordinates [count * n^dim, dim] and weight x det J of the n^dim
    Gauss points of elements first .. first+count-1 (x fastest, element-major)."""
    dim, o = mesh.dim, mesh._order
    x1, w1 = np.polynomial.legendre.leggauss(n_gauss)
    q = np.arange(n_gauss ** dim)
    qi = [q % n_gauss, (q // n_gauss) % n_gauss] + ([q // (n_gauss * n_gauss)] if dim == 3 else [])
    w = np.prod([w1[qi[d]] for d in range(dim)], axis=0)
    e = np.arange(first, first + count)
    r = mesh.elementRes
    ei = [e % r[0], (e // r[0]) % r[1]] + ([e // (r[0] * r[1])] if dim == 3 else [])
    xg = np.empty((count, len(q), dim))
    det = np.ones(count)
    for d in range(dim):
        lo = mesh._axes[d][ei[d] * o]
        hi = mesh._axes[d][(ei[d] + 1) * o]
        xg[:, :, d] = lo[:, None] + (x1[qi[d]][None, :] + 1.0) * 0.5 * (hi - lo)[:, None]
        det *= (hi - lo) / 2.0
    return xg.reshape(-1, dim), (det[:, None] * w[None, :]).reshape(-1)


class _SubMesh:
    """The pressure mesh: dQ0 (one node per element at its centroid) or dPc1
    (three per element in 2D, four in 3D: the coefficients of the linear bases
    of BilinearInnerElType.c:169-179 and TrilinearInnerElType.c:202-215)."""

    def __init__(self, mesh):
        self.parent = mesh
        self.dim = mesh.dim
        self.elementType = "DQ0" if mesh._porder == 0 else "DPC1"
        self._npn = 1 if mesh._porder == 0 else (3 if mesh.dim == 2 else 4)
        self.nodesGlobal = mesh.elementsGlobal * self._npn
        self.elementsGlobal = mesh.elementsGlobal
        self.elementRes = mesh.elementRes

    @property
    def data(self):
        o = self.parent._order
        ax = [0.5 * (a[o::o] + a[:-o:o]) for a in self.parent._axes]
        g = np.meshgrid(*ax, indexing="ij")
        c = np.stack([a.transpose().ravel() for a in g], axis=1)
        return np.repeat(c, self._npn, axis=0)

    def add_variable(self, nodeDofCount, dataType="double", **kwargs):
        return MeshVariable(self, nodeDofCount, dataType)


class _SpecialSets(dict):
    """MinI/MaxI/MinJ/MaxJ(/MinK/MaxK) vertex sets and aliases (P/mesh/_mesh.py:1140-1158).
    Each lookup returns a new set, as the reference builds one per call, so that
    editing a returned set leaves the mesh's own sets unchanged."""

    def __init__(self, mesh):
        super().__init__()
        (ii, nn), dim = mesh._node_grid(), mesh.dim
        N = mesh.nodesGlobal
        names = [("MinI_VertexSet", "Left_VertexSet", 0, 0), ("MaxI_VertexSet", "Right_VertexSet", 0, 1),
                 ("MinJ_VertexSet", "Bottom_VertexSet", 1, 0), ("MaxJ_VertexSet", "Top_VertexSet", 1, 1)]
        if dim == 3:
            names += [("MinK_VertexSet", "Front_VertexSet", 2, 0), ("MaxK_VertexSet", "Back_VertexSet", 2, 1)]
        allw = FeMesh_IndexSet(mesh, 0, N)
        for a, b, d, side in names:
            sel = np.where(ii[d] == (0 if side == 0 else nn[d] - 1))[0]
            s = FeMesh_IndexSet(mesh, 0, N, sel)
            self[a] = s
            self[b] = s
            allw = allw + s
        self["AllWalls_VertexSet"] = allw
        self["Empty"] = FeMesh_IndexSet(mesh, 0, N)

    def __getitem__(self, key):
        return copy.deepcopy(dict.__getitem__(self, key))


class MeshVariable:
    """Nodal field with ``nodeDofCount`` components (host ``data`` + device mirror)."""

    def __init__(self, mesh, nodeDofCount, dataType="double", **kwargs):
        if dataType != "double":
            raise ValueError("only 'double' mesh variables are supported")
        self.mesh = mesh
        self.nodeDofCount = int(nodeDofCount)
        self._data = _core.host_array((mesh.nodesGlobal, self.nodeDofCount), np.float64)
        self._dev = None

    @property
    def data(self):
        return self._data

    @data.setter
    def data(self, v):
        self._data[...] = v

    @property
    def dataType(self):
        return "double"

    def copy(self, deepcopy=False):
        """A new variable on the same mesh with the same components; with
        deepcopy the data too (P/mesh/_meshvariable.py:613-660)."""
        new = MeshVariable(self.mesh, self.nodeDofCount, self.dataType)
        if deepcopy:
            new.data[...] = self._data
        return new

    def syncronise(self):
        """Shadow-node synchronisation: a single-process mesh has no shadows."""
        return None

    def _primary(self):
        return self.mesh if isinstance(self.mesh, FeMesh_Cartesian) else self.mesh.parent

    def _to_device(self):
        ctx = self._primary().ctx
        host = torch.from_numpy(np.ascontiguousarray(self._data).reshape(-1))
        if self._dev is None or self._dev.shape != host.shape:
            self._dev = torch.empty(host.shape, dtype=host.dtype, device=ctx.device)
        self._dev.copy_(host)
        return self._dev

    def _from_device(self):
        if self._data.flags.c_contiguous:
            torch.from_numpy(self._data.reshape(-1)).copy_(self._dev)
        else:
            self._data[...] = self._dev.cpu().numpy().reshape(self._data.shape)

    def _as_function(self):
        return _fn._MeshVar(self)

    def _interpolate_grad(self, coords):
        """Global gradients at points: [n, k*dim], row-major (d v_i / d x_j at i*dim + j)."""
        if not isinstance(self.mesh, FeMesh_Cartesian):
            raise ValueError("gradients are provided for velocity-mesh variables")
        ctx = self.mesh.ctx
        _, g = ctx.interpolate_field(coords.contiguous(), self._to_device(), self.nodeDofCount, grad=True)
        return g.reshape(g.shape[0], -1)

    @property
    def fn_gradient(self):
        """Function of the gradient field (P/mesh/_meshvariable.py:184-225): [dT/dx, dT/dy(, dT/dz)]
        for a scalar, the row-major tensor [dv_x/dx, dv_x/dy, ..., dv_z/dz] for a vector."""
        return _fn._MeshGrad(self)

    def evaluate(self, inputData=None, inputType=None):
        return self._as_function().evaluate(inputData, inputType)

    def evaluate_global(self, inputData, inputType=None):
        return self._as_function().evaluate_global(inputData, inputType)

    def _interpolate(self, coords):
        """Field values at global points (device tensor [n, dim] -> [n, k])."""
        ctx = self._primary().ctx
        if isinstance(self.mesh, FeMesh_Cartesian):
            dev = self._to_device()
            return ctx.interpolate_field(coords.contiguous(), dev, self.nodeDofCount)[0]
        own = ctx.locate(coords.contiguous()).long()
        vals = torch.from_numpy(self._data).to(ctx.device)
        npn = self.mesh._npn
        if npn == 1:
            return vals[own.clamp(max=vals.shape[0] - 1)]
        # dPc1: sum_k p_k M_k(xi) at the points' local coordinates
        pm = self._primary()
        el = own.clamp(max=pm.elementsGlobal - 1)
        r = pm.elementRes
        ij = [el % r[0], (el // r[0]) % r[1]] + ([el // (r[0] * r[1])] if pm.dim == 3 else [])
        xi = []
        for d in range(pm.dim):
            corners = torch.from_numpy(np.ascontiguousarray(pm._axes[d][:: pm._order])).to(ctx.device)
            lo, hi = corners[ij[d]], corners[ij[d] + 1]
            xi.append(2.0 * (coords[:, d] - lo) / (hi - lo) - 1.0)
        if pm.dim == 2:
            M = torch.stack([-xi[0] - 0.5 * xi[1] + 0.25, xi[0] - 0.5 * xi[1] + 0.25, xi[1] + 0.5], 1)
        else:
            x, y, z = xi
            M = torch.stack([-4.0 * x - 20.0 * y + 12.0 * z + 3.0, 16.0 * x - 64.0 * y + 60.0 * z + 6.0,
                             36.0 * y - 36.0 * z, -12.0 * x + 48.0 * y - 36.0 * z], 1) / 9.0
        return (vals.view(-1, npn)[el] * M).sum(1, keepdim=True)

    # -- checkpointing (P/mesh/_meshvariable.py:227-620) ----------------------
    def save(self, filename, meshHandle=None, units=None, **kwargs):
        """Write ``data`` to an HDF5 file (dataset ``data`` [nodes, components];
        attributes units, elementType, ``kwargs`` as strings, and ``mesh``, the
        path of the linked mesh file when ``meshHandle`` is given).  Returns a
        ``SavedFileData``."""
        if not isinstance(filename, str):
            raise TypeError("Expected 'filename' to be provided as a string")
        if units is not None:
            raise NotImplementedError("saving with units (dimensional scaling) is not supported")
        attrs = {str(k): str(v) for k, v in kwargs.items()}
        attrs["units"] = "None"
        attrs["elementType"] = np.bytes_(self.mesh.elementType.encode())
        if meshHandle is not None:
            if not isinstance(meshHandle, (str, _utils.SavedFileData)):
                raise TypeError("Expected 'meshHandle' to be of type 'uw.utils.SavedFileData'")
            mfile = meshHandle if isinstance(meshHandle, str) else meshHandle.filename
            if not os.path.exists(mfile):
                raise ValueError("You are trying to link against the mesh file '%s' that does not appear to exist."
                                 % mfile)
            attrs["mesh"] = os.path.abspath(mfile)
        _h5.write(filename, {"data": self._data}, attrs)
        return _utils.SavedFileData(self, filename)

    def load(self, filename, interpolate=False):
        """Read ``data`` saved by ``save``.  With ``interpolate=True`` a field
        saved on a different resolution of the same element type is evaluated
        at this variable's nodes (the mesh file linked at save time gives the
        source mesh)."""
        if not isinstance(filename, str):
            raise TypeError("Expected 'filename' to be provided as a string")
        with _h5.File(filename) as f:
            d = f["data"]
            link = f.attrs.get("mesh")
            if link is None and "mesh" in f.links:      # an external link, as h5py writes it
                link = f.links["mesh"][0]
                if not os.path.isabs(link):
                    link = os.path.join(os.path.dirname(os.path.abspath(filename)), link)
        if d.ndim != 2 or d.shape[1] != self.nodeDofCount:
            raise RuntimeError("Can't load hdf5 '%s', incompatible data shape" % filename)
        if d.shape[0] == self._data.shape[0]:
            self._data[...] = d
            return
        if not interpolate:
            raise RuntimeError("Provided data file appears to be for a different resolution MeshVariable.\n"
                               "Set 'interpolate=True' to interpolate it onto this variable's nodes.")
        if not isinstance(self.mesh, FeMesh_Cartesian):
            raise NotImplementedError("interpolated loading is provided for velocity-mesh variables")
        if link is None:
            raise RuntimeError("'%s' has no linked mesh file to interpolate from" % filename)
        link = link.decode() if isinstance(link, bytes) else str(link)
        with _h5.File(link) as f:
            a = f.attrs
            res = tuple(int(r) for r in a["mesh resolution"])
            lo = tuple(float(x) for x in a["min"])
            hi = tuple(float(x) for x in a["max"])
            et = a["elementType"]
        et = et.decode() if isinstance(et, bytes) else str(et)
        src = FeMesh_Cartesian("Q1/dQ0" if et.upper() == "Q1" else "Q2/dPc1", res, lo, hi)
        if src.nodesGlobal != d.shape[0]:
            raise RuntimeError("the linked mesh file does not match the saved field")
        var = MeshVariable(src, self.nodeDofCount)
        var.data[...] = d
        pts = torch.from_numpy(np.ascontiguousarray(self.mesh.data)).to(src.ctx.device)
        self._data[...] = var._interpolate(pts).cpu().numpy().reshape(self._data.shape)

    def xdmf(self, filename, fieldSavedData, varname, meshSavedData, meshname, modeltime=0.):
        """Write an XDMF file describing the saved field on the saved mesh."""
        if not isinstance(varname, str):
            raise ValueError("'varname' must be of type str")
        if not isinstance(meshname, str):
            raise ValueError("'meshname' must be of type str")
        if not isinstance(filename, str):
            raise ValueError("'filename' must be of type str")
        if not isinstance(meshSavedData, _utils.SavedFileData):
            raise ValueError("'meshSavedData' must be of type SavedFileData")
        if not isinstance(fieldSavedData, _utils.SavedFileData):
            raise ValueError("'fieldSavedData' must be of type SavedFileData")
        if not isinstance(modeltime, (int, float)):
            raise ValueError("'modeltime' must be of type int or float")
        if self._primary() is not meshSavedData.pyobj:
            raise RuntimeError("'meshSavedData file doesn't correspond to the object's mesh")
        if not filename.lower().endswith(".xdmf"):
            filename += ".xdmf"
        text = (_utils._xdmf_header() + _utils._mesh_grid(meshSavedData, meshname, float(modeltime)) +
                _utils._field(fieldSavedData, varname) + _utils._xdmf_footer())
        with open(filename, "w") as fh:
            fh.write(text)

    def __add__(self, o): return self._as_function() + o
    def __radd__(self, o): return o + self._as_function()
    def __mul__(self, o): return self._as_function() * o
    def __rmul__(self, o): return self._as_function() * o
    def __sub__(self, o): return self._as_function() - o
    def __getitem__(self, i): return self._as_function()[i]
