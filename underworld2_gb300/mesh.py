"""Regular Cartesian FE meshes and mesh variables (``uw.mesh`` subset).

Mirrors ``FeMesh_Cartesian`` / ``MeshVariable`` of the reference
(P/mesh/_mesh.py:1105-1160, P/mesh/_meshvariable.py) for Q1/dQ0 meshes:
node numbering x-fastest, element numbering x-fastest, node coordinates
``min + (i/n)*(max-min)`` (L/StgDomain/Mesh/src/CartesianGenerator.c:2003-2036).
``MeshVariable.data`` is a host numpy array; the library copies it to the
device when a solve or an advection reads it and writes results back in place.
"""
import re

import numpy as np
import torch

from . import _core
from . import function as _fn


class IndexSet:
    """A set of node indices (``uw.container.IndexSet`` subset)."""

    def __init__(self, size, indices=()):
        self.size = int(size)
        self._set = np.unique(np.asarray(list(indices) if not isinstance(indices, np.ndarray) else indices,
                                         dtype=np.int64))

    @property
    def data(self):
        return self._set.copy()

    def __add__(self, other):
        return IndexSet(max(self.size, other.size), np.union1d(self._set, other._set))

    def __len__(self):
        return len(self._set)

    def __iter__(self):
        return iter(self._set.tolist())

    def __contains__(self, i):
        return int(i) in set(self._set.tolist())

    def __repr__(self):
        return "IndexSet(%s)" % self._set.tolist()


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
        elif types[0] == "Q2" and len(types) > 1 and types[1] == "DPC1":
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

    def add_variable(self, nodeDofCount, dataType="double", **kwargs):
        return MeshVariable(self, nodeDofCount, dataType)

    def _node_grid(self):
        n = [r * self._order + 1 for r in self.elementRes]
        idx = np.arange(self.nodesGlobal)
        out = [idx % n[0], (idx // n[0]) % n[1]]
        if self.dim == 3:
            out.append(idx // (n[0] * n[1]))
        return out, n


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
    """MinI/MaxI/MinJ/MaxJ(/MinK/MaxK) vertex sets and aliases (P/mesh/_mesh.py:1140-1158)."""

    def __init__(self, mesh):
        super().__init__()
        (ii, nn), dim = mesh._node_grid(), mesh.dim
        N = mesh.nodesGlobal
        names = [("MinI_VertexSet", "Left_VertexSet", 0, 0), ("MaxI_VertexSet", "Right_VertexSet", 0, 1),
                 ("MinJ_VertexSet", "Bottom_VertexSet", 1, 0), ("MaxJ_VertexSet", "Top_VertexSet", 1, 1)]
        if dim == 3:
            names += [("MinK_VertexSet", "Front_VertexSet", 2, 0), ("MaxK_VertexSet", "Back_VertexSet", 2, 1)]
        allw = IndexSet(N)
        for a, b, d, side in names:
            sel = np.where(ii[d] == (0 if side == 0 else nn[d] - 1))[0]
            s = IndexSet(N, sel)
            self[a] = s
            self[b] = s
            allw = allw + s
        self["AllWalls_VertexSet"] = allw
        self["Empty"] = IndexSet(N)


class MeshVariable:
    """Nodal field with ``nodeDofCount`` components (host ``data`` + device mirror)."""

    def __init__(self, mesh, nodeDofCount, dataType="double", **kwargs):
        if dataType != "double":
            raise ValueError("only 'double' mesh variables are supported")
        self.mesh = mesh
        self.nodeDofCount = int(nodeDofCount)
        self._data = np.zeros((mesh.nodesGlobal, self.nodeDofCount))
        self._dev = None

    @property
    def data(self):
        return self._data

    @data.setter
    def data(self, v):
        self._data[...] = v

    def _primary(self):
        return self.mesh if isinstance(self.mesh, FeMesh_Cartesian) else self.mesh.parent

    def _to_device(self):
        ctx = self._primary().ctx
        t = torch.from_numpy(np.ascontiguousarray(self._data).ravel()).to(ctx.device)
        if self._dev is None or self._dev.shape != t.shape:
            self._dev = t.clone()
        else:
            self._dev.copy_(t)
        return self._dev

    def _from_device(self):
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

    def __add__(self, o): return self._as_function() + o
    def __radd__(self, o): return o + self._as_function()
    def __mul__(self, o): return self._as_function() * o
    def __rmul__(self, o): return self._as_function() * o
    def __sub__(self, o): return self._as_function() - o
    def __getitem__(self, i): return self._as_function()[i]
