"""Particle swarms on the GPU (``uw.swarm`` subset).

The particle state -- coordinates, owning element and the per-element cell
tables -- lives on the device; swarm variables are arrays indexed by particle.
Particles are deleted and created with the reference's array semantics
(escaped-particle removal, population control), which reorder the particle
index; swarm-variable rows follow their particles.
Reference: P/swarm/_swarm.py, P/swarm/_swarmabstract.py, P/swarm/layouts.py,
P/swarm/_integration_swarm.py, P/swarm/_population_control.py.
"""
import contextlib
import os

import numpy as np
import torch

from . import _core
from . import function as _fn
from . import h5 as _h5
from . import utils as _utils

# Park-Miller stream state shared by every random layout, as in
# L/StgDomain/Swarm/src/Random.c (one static seed for the process).
_RNG = {"state": _core.rng_seed(13)}


class SwarmVariable:
    """Per-particle data, host ``data`` array with a device mirror."""

    def __init__(self, swarm, dataType, count):
        if dataType not in ("double", "float", "int", "char", "short", "long"):
            raise ValueError("unsupported dataType %r" % dataType)
        self.swarm = swarm
        self.dataType = dataType
        self.count = int(count)
        np_dt = {"double": np.float64, "float": np.float32, "int": np.int32, "char": np.int8,
                 "short": np.int16, "long": np.int64}[dataType]
        self._data = np.zeros((swarm.particleLocalCount, self.count), dtype=np_dt)
        self._dev = None
        self._dirty = True

    @property
    def data(self):
        self._dirty = True
        return self._data

    def _resize(self, n):
        old = self._data
        self._data = np.zeros((n, self.count), dtype=old.dtype)
        self._data[: min(n, len(old))] = old[: min(n, len(old))]
        self._dirty = True

    def _device_data(self):
        if self._dirty or self._dev is None:
            self._dev = torch.from_numpy(np.ascontiguousarray(self._data)).to(self.swarm.mesh.ctx.device)
            self._dirty = False
        return self._dev

    def _as_function(self):
        return _fn._SwarmVar(self)

    # -- checkpointing (P/swarm/_swarmvariable.py:244-600) --------------------
    def save(self, filename, collective=False, swarmHandle=None, units=None, **kwargs):
        """Write ``data`` to an HDF5 file (dataset ``data`` [particles,
        components]; attributes proc_offset, units, ``kwargs`` as strings, and
        ``swarm``, the path of the linked swarm file when ``swarmHandle`` is
        given).  Returns a ``SavedFileData``."""
        if not isinstance(filename, str):
            raise TypeError("'filename' parameter must be of type 'str'")
        if units is not None:
            raise NotImplementedError("saving with units (dimensional scaling) is not supported")
        attrs = {"proc_offset": np.array([self.swarm.particleLocalCount], dtype=np.int64), "units": "None"}
        if swarmHandle is not None:
            if not isinstance(swarmHandle, (str, _utils.SavedFileData)):
                raise TypeError("Expected 'swarmHandle' to be of type 'uw.utils.SavedFileData'")
            sfile = swarmHandle if isinstance(swarmHandle, str) else swarmHandle.filename
            if not os.path.exists(sfile):
                raise ValueError("You are trying to link against the swarm file '%s' that does not appear to exist."
                                 % sfile)
            attrs["swarm"] = os.path.abspath(sfile)
        attrs.update({str(k): str(v) for k, v in kwargs.items()})
        _h5.write(filename, {"data": self._data}, attrs)
        return _utils.SavedFileData(self, filename)

    def load(self, filename, collective=False):
        """Read ``data`` saved by ``save`` into the particles of a swarm that was
        itself loaded from its checkpoint (``Swarm.load``), row by saved index."""
        if not isinstance(filename, str):
            raise TypeError("'filename' parameter must be of type 'str'")
        sw = self.swarm
        if getattr(sw, "_checkpointMapsToState", None) != sw.stateId:
            raise RuntimeError("'Swarm' associate with this 'SwarmVariable' does not appear to be in the correct "
                               "state.\nPlease ensure that you have loaded the swarm prior to loading any swarm "
                               "variables.")
        with _h5.File(filename) as f:
            d = f["data"]
        if d.shape[1] != self._data.shape[1]:
            raise RuntimeError("Cannot load file data on current swarm. Data in file '%s' has %d components, the "
                               "variable has %d" % (filename, d.shape[1], self._data.shape[1]))
        if d.shape[0] != sw._checkpointCount:
            raise RuntimeError("It appears that the swarm has %d particles, but provided h5 file has %d data points."
                               % (sw._checkpointCount, d.shape[0]))
        first = sw._checkpointFirst
        self._data[first:first + len(sw._local2globalMap)] = d[sw._local2globalMap]
        self._dirty = True

    def xdmf(self, filename, varSavedData, varname, swarmSavedData, swarmname, modeltime=0.):
        """Write an XDMF file describing the saved variable on the saved swarm."""
        if not isinstance(varname, str):
            raise ValueError("'varname' must be of type str")
        if not isinstance(swarmname, str):
            raise ValueError("'swarmname' must be of type str")
        if not isinstance(filename, str):
            raise ValueError("'filename' must be of type str")
        if not isinstance(swarmSavedData, _utils.SavedFileData):
            raise ValueError("'swarmSavedData' must be of type SavedFileData")
        if not isinstance(varSavedData, _utils.SavedFileData):
            raise ValueError("'varSavedData' must be of type SavedFileData")
        if not isinstance(modeltime, (int, float)):
            raise ValueError("'modeltime' must be of type int or float")
        if not filename.lower().endswith(".xdmf"):
            filename += ".xdmf"
        text = (_utils._xdmf_header() + _utils._swarm_grid(swarmSavedData, swarmname, float(modeltime)) +
                _utils._swarmvar(varSavedData, varname) + _utils._xdmf_footer())
        with open(filename, "w") as fh:
            fh.write(text)

    def __add__(self, o): return self._as_function() + o
    def __radd__(self, o): return o + self._as_function()
    def __mul__(self, o): return self._as_function() * o
    def __rmul__(self, o): return self._as_function() * o
    def __sub__(self, o): return self._as_function() - o
    def __rsub__(self, o): return o - self._as_function()
    def __truediv__(self, o): return self._as_function() / o
    def __lt__(self, o): return self._as_function() < o
    def __gt__(self, o): return self._as_function() > o
    def __le__(self, o): return self._as_function() <= o
    def __ge__(self, o): return self._as_function() >= o


class _CoordVariable:
    def __init__(self, swarm):
        self.swarm = swarm

    @property
    def data(self):
        return self.swarm.data


class _OwnerVariable:
    def __init__(self, swarm):
        self.swarm = swarm

    @property
    def data(self):
        return self.swarm._owner.cpu().numpy().reshape(-1, 1)


class Swarm:
    """A particle swarm supported by a mesh (P/swarm/_swarm.py:106)."""

    def __init__(self, mesh, particleEscape=False, **kwargs):
        self.mesh = mesh
        self.particleEscape = particleEscape
        self.dim = mesh.dim
        self._x = None
        self._owner = None
        self._off = None
        self._lst = None
        self._variables = []
        self._state = 0
        self._host_x = None
        self._writable = False
        self._voronoi = None
        self.particleCoordinates = _CoordVariable(self)
        self.owningCell = _OwnerVariable(self)

    # -- size and data ---------------------------------------------------------
    @property
    def particleLocalCount(self):
        return 0 if self._x is None else int(self._x.shape[0])

    @property
    def particleGlobalCount(self):
        return self.particleLocalCount

    @property
    def stateId(self):
        return self._state

    @property
    def data(self):
        if self._host_x is None:
            self._host_x = np.zeros((0, self.dim)) if self._x is None else np.array(self._x.cpu().numpy(), copy=True)
        self._host_x.flags.writeable = self._writable
        return self._host_x

    def add_variable(self, dataType, count):
        v = SwarmVariable(self, dataType, count)
        self._variables.append(v)
        return v

    # -- checkpointing (P/swarm/_swarm.py:226-420) ----------------------------
    def save(self, filename, collective=False, units=None, **kwargs):
        """Write the particle coordinates to an HDF5 file (dataset ``data``
        [particles, dim]; attributes proc_offset, units and ``kwargs`` as
        strings).  Returns a ``SavedFileData``."""
        if not isinstance(filename, str):
            raise TypeError("Expected 'filename' to be provided as a string")
        if units is not None:
            raise NotImplementedError("saving with units (dimensional scaling) is not supported")
        attrs = {"proc_offset": np.array([self.particleLocalCount], dtype=np.int64), "units": "None"}
        attrs.update({str(k): str(v) for k, v in kwargs.items()})
        _h5.write(filename, {"data": self.data}, attrs)
        return _utils.SavedFileData(self, filename)

    def load(self, filename, collective=False, try_optimise=True):
        """Add the particles saved in ``filename`` (coordinates outside the mesh
        are skipped), in file order, and record which saved row each one came
        from so that swarm variables saved with the swarm can be loaded."""
        if not isinstance(filename, str):
            raise TypeError("Expected 'filename' to be provided as a string")
        with _h5.File(filename) as f:
            d = f["data"]
        if d.ndim != 2 or d.shape[1] != self.dim:
            raise RuntimeError("Cannot load file data on current swarm. Data in file '%s' has %d components, the "
                               "particle coordinates have %d" % (filename, d.shape[1], self.dim))
        chunk = 20_000_000
        self._checkpointFirst = self.particleLocalCount
        rows = []
        for start in range(0, d.shape[0], chunk):
            ret = self.add_particles_with_coordinates(np.ascontiguousarray(d[start:start + chunk]))
            rows.append(start + np.nonzero(ret >= 0)[0])
        self._local2globalMap = np.concatenate(rows) if rows else np.zeros(0, dtype=np.int64)
        self._checkpointCount = d.shape[0]
        self._checkpointMapsToState = self.stateId

    # -- population ------------------------------------------------------------
    def populate_using_layout(self, layout):
        if self.particleLocalCount > 0:
            raise RuntimeError("Swarm appears to already have particles. \nLayouts can only be used with empty swarms.")
        if not isinstance(layout, _ParticleLayoutAbstract):
            raise TypeError("Provided layout does not appear to be a subclass of ParticleLayout")
        if layout.swarm is not self:
            raise ValueError("The swarm associated with the layout appears to be a different swarm from self.")
        layout._populate()

    def add_particles_with_coordinates(self, coordinatesArray):
        """Adds particles; coordinates outside the mesh are rejected (index -1)."""
        if not isinstance(coordinatesArray, np.ndarray):
            raise TypeError("'coordinateArray' must be provided as a numpy array")
        if coordinatesArray.ndim != 2 or coordinatesArray.shape[1] != self.dim:
            raise ValueError("The 'coordinateArray' must have shape n*dim")
        ctx = self.mesh.ctx
        new = torch.from_numpy(np.ascontiguousarray(coordinatesArray, dtype=np.float64)).to(ctx.device)
        own = ctx.locate(new)
        keep = own < ctx.n_el
        kept = new[keep]
        n0 = self.particleLocalCount
        ret = np.full(len(coordinatesArray), -1, dtype=np.int32)
        ret[keep.cpu().numpy()] = np.arange(n0, n0 + int(keep.sum()), dtype=np.int32)
        if self._x is None or n0 == 0:
            self._set_particles(kept, rebuild=True)
            return ret
        # Swarm_AddParticleToCell: each new particle is appended to its element's
        # table, in array order, after the particles already there
        n_in = int(self._off[-1])
        old_lst = self._lst[:n_in].long()
        old_cells = self._owner.long()[old_lst]
        new_cells = own[keep].long()
        keys = torch.cat([old_cells, new_cells])
        vals = torch.cat([old_lst, torch.arange(n0, n0 + kept.shape[0], device=ctx.device)])
        order = torch.argsort(keys, stable=True)
        counts = torch.bincount(keys, minlength=ctx.n_el)[: ctx.n_el]
        off = torch.zeros(ctx.n_el + 1, dtype=torch.int32, device=ctx.device)
        off[1:] = torch.cumsum(counts, 0).to(torch.int32)
        x = torch.cat([self._x, kept])
        owner = torch.cat([self._owner, own[keep].to(torch.int32)])
        lst = vals[order].to(torch.int32)
        pad = x.shape[0] - lst.shape[0]
        if pad:
            lst = torch.cat([lst, torch.zeros(pad, dtype=torch.int32, device=ctx.device)])
        self._set_particles(x, owner, off, lst.contiguous())
        return ret

    def _set_particles(self, x, owner=None, off=None, lst=None, rebuild=False):
        ctx = self.mesh.ctx
        self._x = x.contiguous()
        if rebuild:
            owner = ctx.locate(self._x)
            # cell tables in particle order (what Swarm_AddParticleToCell produces)
            o = owner.long()
            order = torch.argsort(o, stable=True)
            counts = torch.bincount(o, minlength=ctx.n_el + 1)[: ctx.n_el]
            off = torch.zeros(ctx.n_el + 1, dtype=torch.int32, device=ctx.device)
            off[1:] = torch.cumsum(counts, 0).to(torch.int32)
            n_in = int(off[-1])
            lst = order[:n_in].to(torch.int32).contiguous()
            lst = torch.cat([lst, torch.zeros(self._x.shape[0] - n_in, dtype=torch.int32, device=ctx.device)])
        self._owner, self._off, self._lst = owner, off, lst
        for v in self._variables:
            v._resize(self.particleLocalCount)
        self._host_x = None
        self._toggle_state()

    def _toggle_state(self):
        self._state += 1

    # -- movement --------------------------------------------------------------
    @contextlib.contextmanager
    def deform_swarm(self, update_owners=True):
        """Particle coordinates may be modified inside this context."""
        data = self.data
        self._writable = True
        data.flags.writeable = True
        try:
            yield
        finally:
            self._writable = False
            self._x.copy_(torch.from_numpy(np.ascontiguousarray(self._host_x)).to(self._x.device))
            self._host_x = None
            if update_owners:
                self.update_particle_owners()

    def update_particle_owners(self):
        """Swarm_UpdateAllParticleOwners, then EscapedRoutine_RemoveFromSwarm: particles
        outside the mesh are deleted, and that is an error unless particleEscape is set
        (P/swarm/_swarm.py:613-654)."""
        ctx = self.mesh.ctx
        lost = ctx.update_owners(self._x, self._owner, self._off, self._lst)
        if lost:
            np_new = ctx.pop_plan_escaped(self._owner, self._off, self._lst)
            self._apply_population(np_new, None)
        self._host_x = None
        self._toggle_state()
        if lost and not self.particleEscape:
            raise RuntimeError("Particles appear to have left the domain, but swarm flag `particleEscape` is False. "
                               "Check your velocity field or your particle relocation routines, or set the "
                               "`particleEscape` swarm constructor parameter to True to allow escape.")
        return lost

    def _apply_population(self, np_new, ip_xi):
        """Write the library's pending deletion/creation plan into the particle arrays."""
        x, owner, off, lst, src = self.mesh.ctx.pop_apply(ip_xi, self._x, np_new)
        for v in self._variables:
            v._data = np.ascontiguousarray(v._data[src])
            v._dirty = True
        self._x, self._owner, self._off, self._lst = x, owner, off, lst
        self._host_x = None

    # -- the PIC integration swarm ---------------------------------------------
    @property
    def _voronoi_swarm(self):
        if self._voronoi is None:
            self._voronoi = VoronoiIntegrationSwarm(self)
        return self._voronoi


class VoronoiIntegrationSwarm:
    """Integration points coincident with the material particles, weighted by
    discrete Voronoi cells (P/swarm/_integration_swarm.py:118-145)."""

    def __init__(self, swarm, resolution=15):
        self.swarm = swarm
        self.res = resolution
        self._mapped_state = -1
        self.ip_xi = None
        self.ip_w = None

    def repopulate(self):
        s = self.swarm
        if self._mapped_state == s.stateId:
            return
        ctx = s.mesh.ctx
        self.ip_xi = ctx.pic_map(s._x, s._off, s._lst)
        self.ip_w = ctx.dvc_weights(s._off, self.ip_xi, self.res)
        self._mapped_state = s.stateId

    def global_coords(self):
        """Global position of every integration point (slot order)."""
        s = self.swarm
        ctx = s.mesh.ctx
        off = s._off.long()
        n = int(off[-1])
        slots = torch.arange(n, device=ctx.device)
        el = torch.searchsorted(off[1:], slots, right=True)
        res = ctx.res
        idx = [el % res[0], (el // res[0]) % res[1]] + ([el // (res[0] * res[1])] if ctx.dim == 3 else [])
        out = torch.empty((n, ctx.dim), dtype=torch.float64, device=ctx.device)
        for d in range(ctx.dim):
            ax = torch.from_numpy(ctx.axes[d]).to(ctx.device)
            lo, hi = ax[idx[d]], ax[idx[d] + 1]
            out[:, d] = lo + (self.ip_xi[:n, d] + 1.0) * 0.5 * (hi - lo)
        return out


class PopulationControl:
    """Per-element population control with discrete Voronoi volumes
    (P/swarm/_population_control.py:14-93; PCDVC.c): particles whose Voronoi
    volume fraction of their element exceeds ``splitThreshold`` are split (at
    most ``maxSplits`` per element, the copy placed at the centroid of the
    particle's Voronoi cell), those below ``deleteThreshold`` are deleted (at
    most ``maxDeletions`` per element)."""

    def __init__(self, swarm, deleteThreshold=0.006, splitThreshold=0.25, maxDeletions=0, maxSplits=3,
                 aggressive=False, aggressiveThreshold=0.8, particlesPerCell=None, **kwargs):
        if not isinstance(swarm, Swarm):
            raise TypeError("Provided 'swarm' must be of 'Swarm' class.")
        if not isinstance(deleteThreshold, (int, float)):
            raise TypeError("'deleteThreshold' parameter must of type 'float'.")
        if deleteThreshold < 0.0 or deleteThreshold > 1.0:
            raise ValueError("'deleteThreshold' parameter must take values in [0.,1.].")
        if not isinstance(splitThreshold, (int, float)):
            raise TypeError("'splitThreshold' parameter must of type 'float'.")
        if splitThreshold < 0.0 or splitThreshold > 1.0:
            raise ValueError("'splitThreshold' parameter must take values in [0.,1.].")
        if deleteThreshold > splitThreshold:
            raise ValueError("'deleteThreshold' must be less than 'splitThreshold'.")
        if not isinstance(maxDeletions, int):
            raise TypeError("'maxDeletions' parameter must of type 'int'.")
        if maxDeletions < 0:
            raise ValueError("'maxDeletions' parameter must take non-negative values.")
        if not isinstance(maxSplits, int):
            raise TypeError("'maxSplits' parameter must of type 'int'.")
        if maxSplits < 0:
            raise ValueError("'maxSplits' parameter must take non-negative values.")
        if not isinstance(aggressive, bool):
            raise TypeError("'aggressive' parameter must of type 'bool'.")
        if aggressive:
            raise NotImplementedError("aggressive population control draws from the C library's rand() stream; "
                                      "it is not provided on the GPU path")
        self._swarm = swarm
        self.deleteThreshold, self.splitThreshold = float(deleteThreshold), float(splitThreshold)
        self.maxDeletions, self.maxSplits = maxDeletions, maxSplits
        self.last = None

    def repopulate(self):
        """Split and delete particles; the swarm's state changes (its integration swarm is re-mapped)."""
        s = self._swarm
        if s.particleLocalCount == 0:
            return
        ctx = s.mesh.ctx
        ip_xi = ctx.pic_map(s._x, s._off, s._lst)
        ip_w = ctx.dvc_weights(s._off, ip_xi, 15)
        np_new, ns, nd = ctx.pop_plan_pcdvc(s._owner, s._off, s._lst, ip_w, self.splitThreshold,
                                            self.deleteThreshold, self.maxSplits, self.maxDeletions)
        if ns or nd:
            s._apply_population(np_new, ip_xi)
        self.last = {"splits": ns, "deletions": nd}
        s._toggle_state()


class _ParticleLayoutAbstract:
    def __init__(self, swarm, **kwargs):
        self.swarm = swarm


class PerCellRandomLayout(_ParticleLayoutAbstract):
    """Per-element uniform random layout with the reference's Park-Miller stream
    (P/swarm/layouts.py:186-231, L/StgFEM/Utils/src/MeshParticleLayout.c:194-230).
    Constructing a layout seeds the process-wide stream, as Swarm_Random_Seed does."""

    def __init__(self, swarm, particlesPerCell, seed=13, **kwargs):
        super().__init__(swarm)
        self.particlesPerCell = int(particlesPerCell)
        self.seed = int(seed)
        _RNG["state"] = _core.rng_seed(self.seed)

    def _populate(self):
        ctx = self.swarm.mesh.ctx
        x, owner, off, lst, st = ctx.layout_random(self.particlesPerCell, _RNG["state"])
        _RNG["state"] = st
        self.swarm._set_particles(x, owner, off, lst)


class layouts:
    PerCellRandomLayout = PerCellRandomLayout
