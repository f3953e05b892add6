"""Integrals, checkpoint handles and XDMF descriptions (``uw.utils`` subset).

``SavedFileData`` is what every ``save`` returns (P/utils/_utils.py:207-222).
The XDMF writers describe saved HDF5 files to visualisation tools in the
reference's layout (P/utils/_utils.py:224-554): a uniform grid whose topology
is read from the mesh file's ``en_map`` and geometry from ``vertices``, and
attributes read from a variable file's ``data``.  The element-node map is
stored in lexicographic node order (x fastest); the XDMF topology reorders it
into the corner-then-edge order of the XDMF/VTK cell types through a JOIN of
per-column hyperslabs.
"""
import os

from . import h5


class Integral:
    """Volume or surface integral of a function over a mesh (P/utils/_utils.py:
    38-206): Gauss points (3 per axis on Q1 meshes, 5 on Q2, as
    GaussIntegrationSwarm), weight x det J, the function evaluated on the
    device; a surface integral sums the Gauss points of the faces that lie in
    ``surfaceIndexSet`` (the reference's border swarm and 0.999 indicator mask)
    with the surface Jacobian.  ``evaluate()`` returns one value per function
    component."""

    def __init__(self, fn, mesh=None, integrationType="volume", surfaceIndexSet=None, integrationSwarm=None,
                 **kwargs):
        from .mesh import FeMesh_Cartesian
        import numpy as np
        if not mesh:
            raise ValueError("A mesh object must be provided")
        if not isinstance(mesh, FeMesh_Cartesian):
            raise TypeError("'feMesh' object passed in must be of type 'FeMesh'")
        if integrationType and integrationSwarm:
            raise RuntimeError("Either an 'integrationType' or an 'integrationSwarm' may be provided, but not both.\n"
                               "You may need to set 'integrationType' to None.")
        self._ng = None
        if integrationSwarm is not None:
            from .swarm import GaussIntegrationSwarm
            if not isinstance(integrationSwarm, GaussIntegrationSwarm):
                raise NotImplementedError("integration swarms other than GaussIntegrationSwarm are not supported")
            if integrationSwarm.mesh is not mesh:
                raise ValueError("The integration swarm must live on the provided mesh")
            self._ng = integrationSwarm.particleCount
            integrationType = "volume"
        if not isinstance(integrationType, str):
            raise TypeError("'integrationType' provided must be a string.")
        integrationType = integrationType.lower()
        if integrationType not in ("volume", "surface"):
            raise ValueError("'integrationType' string provided must be either 'volume' or 'surface'.")
        self._mesh = mesh
        self._surface = integrationType == "surface"
        self._node_on = None
        if self._surface:
            if surfaceIndexSet is None:
                raise RuntimeError("For surface integration, you must provide a 'surfaceIndexSet'.")
            idx = np.asarray(surfaceIndexSet.data if hasattr(surfaceIndexSet, "data") else list(surfaceIndexSet),
                             dtype=np.int64)
            walls = set(mesh.specialSets["AllWalls_VertexSet"].data.tolist())
            if any(int(i) not in walls for i in idx):
                raise ValueError("Your surfaceIndexSet appears to contain node(s) which do not belong to the mesh "
                                 "boundary. Surface integration across internal nodes is not currently supported.")
            self._node_on = np.zeros(mesh.nodesGlobal, dtype=bool)
            self._node_on[idx] = True
        self.fn = fn

    @property
    def fn(self):
        return self._fn

    @fn.setter
    def fn(self, fn):
        from . import function as _fn
        f = _fn.Function.convert(fn)
        if not isinstance(f, _fn.Function):
            raise TypeError("'fn' must be of or convertible to 'Function' class.")
        self._fn = f

    def _eval(self, pts, wts, dev, pid=None):
        import torch
        from . import function as _fn
        xt = torch.from_numpy(pts).to(dev)
        mapped = pid is not None
        if pid is None:
            pid = torch.full((xt.shape[0],), -1, dtype=torch.int64, device=dev)
        ectx = _fn.EvalContext(pid, lambda: xt, dev)
        if mapped:
            ectx.map_swarm = self._map_swarm
        v = self._fn.evaluate_at(ectx).to(torch.float64)
        return (v * torch.from_numpy(wts).to(dev)[:, None]).sum(0)

    def _gauss_particles(self, ng):
        """For swarm-variable integrands: the particle each Gauss point reads, the
        nearest of its element (GeneralSwarm_IntegrationPointMap,
        L/PICellerator/MaterialPoints/src/GeneralSwarm.cpp:319-431), element-major."""
        import numpy as np
        import torch
        from .systems import _swarms_in
        swarms = _swarms_in(self._fn)
        if not swarms:
            return None
        if self._surface:
            raise NotImplementedError("surface integrals of swarm variables are not supported")
        if len(swarms) > 1:
            raise NotImplementedError("swarm variables of more than one swarm in one integrand")
        sw = swarms[0]
        if sw.mesh is not self._mesh:
            raise ValueError("the integrand's swarm lives on another mesh")
        if sw._x is None or sw._off is None:
            raise RuntimeError("Error occurred while trying to evaluate swarm variable. This can occur when there "
                               "are no particles found in a given element.")
        x1, _ = np.polynomial.legendre.leggauss(ng)
        dim = self._mesh.dim
        q = np.arange(ng ** dim)
        xi = np.stack([x1[q % ng], x1[(q // ng) % ng]] + ([x1[q // (ng * ng)]] if dim == 3 else []), 1)
        ctx = self._mesh.ctx
        pid = ctx.gauss_nearest(torch.from_numpy(xi), sw._off, sw._lst, sw._x)
        if bool((pid < 0).any()) and _swarms_in(self._fn, variables_only=True):
            raise RuntimeError("Error occurred while trying to evaluate swarm variable. This can occur when there "
                               "are no particles found in a given element. You may wish to add population "
                               "control mechanisms.")
        self._map_swarm = sw
        return pid.long()

    def evaluate(self):
        import numpy as np
        import torch
        from .mesh import _border_points, _volume_points
        dev = torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")
        m = self._mesh
        ng = self._ng or (3 if m._order == 1 else 5)
        if self._surface:
            xg, fac, _, _ = _border_points(m, self._node_on, ng)
            if len(xg) == 0:
                return np.zeros(1)
            return self._eval(xg, fac, dev).cpu().numpy()
        pid = self._gauss_particles(ng)
        if pid is not None:
            dev = pid.device
        nq = ng ** m.dim
        total = None
        step = max(1, (1 << 22) // nq)
        for first in range(0, m.elementsGlobal, step):
            cnt = min(step, m.elementsGlobal - first)
            pts, wts = _volume_points(m, ng, first, cnt)
            part = self._eval(pts, wts, dev, None if pid is None else pid[first * nq:(first + cnt) * nq])
            total = part if total is None else total + part
        return total.cpu().numpy()


class SavedFileData:
    """A saved object and the absolute path of its file."""

    def __init__(self, pyobj, filename):
        self.pyobj = pyobj
        self.filename = os.path.abspath(filename)


# lexicographic element node index -> position in the XDMF/VTK cell ordering
# (corners counter-clockwise from the origin, then mid-edges, then mid-faces:
# -x, +x, -y, +y, -z, +z, then the centre).  Index into the en_map columns.
def _lex(i, j, k=0, n=2):
    return i + n * j + n * n * k


_CELL_ORDER = {
    (2, 1): ("Quadrilateral", [_lex(0, 0), _lex(1, 0), _lex(1, 1), _lex(0, 1)]),
    (3, 1): ("Hexahedron", [_lex(0, 0, 0), _lex(1, 0, 0), _lex(1, 1, 0), _lex(0, 1, 0),
                            _lex(0, 0, 1), _lex(1, 0, 1), _lex(1, 1, 1), _lex(0, 1, 1)]),
    (2, 2): ("Quadrilateral_9", [_lex(i, j, 0, 3) for i, j in
                                 [(0, 0), (2, 0), (2, 2), (0, 2), (1, 0), (2, 1), (1, 2), (0, 1), (1, 1)]]),
    (3, 2): ("Hexahedron_27", [_lex(i, j, k, 3) for i, j, k in
                               [(0, 0, 0), (2, 0, 0), (2, 2, 0), (0, 2, 0), (0, 0, 2), (2, 0, 2), (2, 2, 2), (0, 2, 2),
                                (1, 0, 0), (2, 1, 0), (1, 2, 0), (0, 1, 0), (1, 0, 2), (2, 1, 2), (1, 2, 2), (0, 1, 2),
                                (0, 0, 1), (2, 0, 1), (2, 2, 1), (0, 2, 1),
                                (0, 1, 1), (2, 1, 1), (1, 0, 1), (1, 2, 1), (1, 1, 0), (1, 1, 2), (1, 1, 1)]]),
}

_NUMBER_TYPE = {"f8": ("Float", 8), "f4": ("Float", 4), "i4": ("Int", 4), "i8": ("Int", 8), "i2": ("Int", 2),
                "i1": ("Char", 1), "u1": ("UChar", 1)}


def _xdmf_header():
    return ('<?xml version="1.0" ?>\n'
            '<Xdmf xmlns:xi="http://www.w3.org/2001/XInclude" Version="2.0">\n'
            "<Domain>\n")


def _xdmf_footer():
    return "</Grid>\n</Domain>\n</Xdmf>\n"


def _hyperslab_column(rows, col, ncols, ref, numtype, name=None):
    nm = ' Name="%s"' % name if name else ""
    return ('\t\t<DataItem ItemType="HyperSlab" Dimensions="%d 1"%s>\n'
            '\t\t\t<DataItem Dimensions="3 2" Format="XML"> 0 %d 1 1 %d 1 </DataItem>\n'
            '\t\t\t<DataItem Format="HDF" %s Dimensions="%d %d">%s</DataItem>\n'
            "\t\t</DataItem>\n" % (rows, nm, col, rows, numtype, rows, ncols, ref))


def _mesh_grid(saved_mesh, meshname, time):
    """Grid, time, topology and geometry of a saved mesh file."""
    mesh = saved_mesh.pyobj
    ref = os.path.basename(saved_mesh.filename)
    n_el, n_nodes, dim = mesh.elementsGlobal, mesh.nodesGlobal, mesh.dim
    ctype, order = _CELL_ORDER[(dim, mesh._order)]
    nen = len(order)
    out = '<Grid Name="FEM_Mesh_%s">\n\n\t<Time Value="%s" />\n\n' % (meshname, time)
    out += '\t<Topology Type="%s" NumberOfElements="%d">\n' % (ctype, n_el)
    out += '\t\t<DataItem ItemType="Function" Dimensions="%d %d" Function="JOIN(%s)">\n' % (
        n_el, nen, ", ".join("$%d" % c for c in order))
    for c in range(nen):
        out += _hyperslab_column(n_el, c, nen, "%s:/en_map" % ref, 'NumberType="Int"', "C%d" % c)
    out += "\t\t</DataItem>\n\t</Topology>\n"
    ft = 'NumberType="Float" Precision="8"'
    out += '\t<Geometry Type="XYZ">\n'
    if dim == 2:
        out += '\t\t<DataItem ItemType="Function" Dimensions="%d 3" Function="JOIN($0, $1, 0*$1)">\n' % n_nodes
        out += _hyperslab_column(n_nodes, 0, 2, "%s:/vertices" % ref, ft, "XCoords")
        out += _hyperslab_column(n_nodes, 1, 2, "%s:/vertices" % ref, ft, "YCoords")
        out += "\t\t</DataItem>\n"
    else:
        out += '\t<DataItem Format="HDF" %s Dimensions="%d 3">%s:/vertices</DataItem>\n' % (ft, n_nodes, ref)
    out += "\t</Geometry>\n"
    return out


def _attribute(varname, numtype, center, count, dof, ref):
    """XDMF attribute for ``count`` rows of ``dof`` components in ``ref:/data``."""
    src = '\t\t\t<DataItem Format="HDF" %s Dimensions="%d %d">%s:/data</DataItem>\n' % (numtype, count, dof, ref)
    if dof in (1, 3, 9):
        kind = {1: "Scalar", 3: "Vector", 9: "Tensor"}[dof]
        return ('\t<Attribute Type="%s" Center="%s" Name="%s">\n%s\t</Attribute>\n' % (kind, center, varname, src))
    if dof == 2:
        out = '\t<Attribute Type="Vector" Center="%s" Name="%s">\n' % (center, varname)
        out += '\t<DataItem ItemType="Function"  Dimensions="%d 3" Function="JOIN($0, $1, 0*$1)">\n' % count
        out += _hyperslab_column(count, 0, 2, "%s:/data" % ref, numtype, "XValue")
        out += _hyperslab_column(count, 1, 2, "%s:/data" % ref, numtype, "YValue")
        return out + "\t</DataItem>\n\t</Attribute>\n"
    if dof == 6:
        # symmetric tensor stored (00, 11, 22, 01, 02, 12); XDMF Tensor6 wants (00, 01, 02, 11, 12, 22)
        out = '\t<Attribute Type="Tensor6" Center="%s" Name="%s">\n' % (center, varname)
        out += '\t<DataItem ItemType="Function"  Dimensions="%d 6" Function="JOIN($0, $3, $4, $1, $5, $2)">\n' % count
        for c in range(6):
            out += _hyperslab_column(count, c, 6, "%s:/data" % ref, numtype, "x%d" % c)
        return out + "\t</DataItem>\n\t</Attribute>\n"
    out = ""
    for c in range(dof):
        out += '\t<Attribute Type="Scalar" Center="%s" Name="%s-Component-%d">\n' % (center, varname, c)
        out += _hyperslab_column(count, c, dof, "%s:/data" % ref, numtype)
        out += "\t</Attribute>\n"
    return out


def _number_type(dtype):
    t, p = _NUMBER_TYPE[dtype.str[1:]]
    return 'NumberType="%s" Precision="%d"' % (t, p)


def _field(saved_var, varname):
    var = saved_var.pyobj
    ref = os.path.basename(saved_var.filename)
    mesh = var._primary()
    count, dof = var.data.shape
    ft = 'NumberType="Float" Precision="8"'
    if count == mesh.nodesGlobal:
        return _attribute(varname, ft, "Node", count, dof, ref)
    if count == mesh.elementsGlobal:
        return _attribute(varname, ft, "Cell", count, dof, ref)
    # discontinuous pressure: the element average of its coefficient rows
    npn = count // mesh.elementsGlobal
    n_el = mesh.elementsGlobal
    out = '\t<Attribute Type="Scalar" Center="Cell" Name="%s">\n' % varname
    out += '\t\t<DataItem ItemType="Function" Dimensions="%d 1" Function="%s">\n' % (
        n_el, "+".join("$%d/%d" % (k, npn) for k in range(npn)))
    for k in range(npn):
        out += ('\t\t\t<DataItem ItemType="HyperSlab" Dimensions="%d 1" Name="P%d">\n'
                '\t\t\t\t<DataItem Dimensions="3 2" Format="XML"> 0 0 %d 1 %d 1 </DataItem>\n'
                '\t\t\t\t\t<DataItem Format="HDF" %s Dimensions="%d 1">%s:/data</DataItem>\n'
                "\t\t\t</DataItem>\n" % (n_el, k, npn, n_el, ft, count, ref))
    return out + "\t\t</DataItem>\n\t</Attribute>\n"


def _swarm_grid(saved_swarm, swarmname, time):
    swarm = saved_swarm.pyobj
    ref = os.path.basename(saved_swarm.filename)
    with h5.File(saved_swarm.filename) as f:
        if "data" not in f:
            raise RuntimeError("Can't find 'data' in file '%s'." % saved_swarm.filename)
        count = f["data"].shape[0]
    dim = swarm.mesh.dim
    out = '<Grid Name="%s" GridType="Uniform">\n\n\t<Time Value="%s" />\n\n' % (swarmname, time)
    out += '\t<Topology Type="POLYVERTEX" NodesPerElement="%d"> </Topology>\n' % count
    out += '\t\t<Geometry Type="%s">\n' % ("XY" if dim == 2 else "XYZ")
    out += ('\t\t\t<DataItem Format="HDF" NumberType="Float" Precision="8" Dimensions="%d %d">%s:/data</DataItem>\n'
            % (count, dim, ref))
    return out + "\t\t</Geometry>\n"


def _swarmvar(saved_var, varname):
    var = saved_var.pyobj
    ref = os.path.basename(saved_var.filename)
    with h5.File(saved_var.filename) as f:
        if "data" not in f:
            raise RuntimeError("Can't find 'data' in file '%s'." % saved_var.filename)
        count = f["data"].shape[0]
    return _attribute(varname, _number_type(var.data.dtype), "Node", count, var.data.shape[1], ref)


def _nps_2norm(v, comm=None):
    """2-norm of a numpy vector (P/utils/_utils.py:645-672); one process holds it all."""
    import numpy as np
    v = np.asarray(v, dtype=np.float64)
    return float(np.sqrt(np.sum(v * v)))
