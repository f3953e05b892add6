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
        self._data = _core.host_array((swarm.particleLocalCount, self.count), np_dt)
        self._dev = None
        self._dirty = True

    @property
    def data(self):
        self._dirty = True
        return self._data

    def copy(self, deepcopy=False):
        """A new variable of the same type and count on the same swarm; with
        deepcopy the data too (P/swarm/_swarmvariable.py)."""
        new = self.swarm.add_variable(self.dataType, self.count)
        if deepcopy:
            new.data[...] = self._data
        return new

    def _resize(self, n):
        old = self._data
        self._data = _core.host_array((n, self.count), old.dtype)
        self._data[: min(n, len(old))] = old[: min(n, len(old))]
        self._dirty = True

    def _set_rows(self, rows):
        """Replace the data by the given rows (a population change), in page-locked memory."""
        new = _core.host_array(rows.shape, self._data.dtype)
        new[...] = rows
        self._data = new
        self._dirty = True

    def _device_data(self):
        if self._dirty or self._dev is None:
            host = torch.from_numpy(np.ascontiguousarray(self._data))
            if self._dev is None or self._dev.shape != host.shape or self._dev.dtype != host.dtype:
                self._dev = torch.empty(host.shape, dtype=host.dtype, device=self.swarm.mesh.ctx.device)
            self._dev.copy_(host)
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

    def evaluate(self, inputData=None, inputType=None):
        """Values at the swarm's particles, at another swarm's or mesh's points or at
        coordinates (the nearest particle's value), as a Function
        (P/function/_function.py:808-930)."""
        return self._as_function().evaluate(inputData, inputType)

    def evaluate_global(self, inputData, inputType=None):
        return self._as_function().evaluate_global(inputData, inputType)

    def __getitem__(self, i): return self._as_function()[i]
    def __neg__(self): return -self._as_function()
    def __pow__(self, o): return self._as_function() ** o
    def __rtruediv__(self, o): return o / self._as_function()
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
        self._host_x = None          # page-locked host mirror of the coordinates (kept between uses)
        self._host_valid = False     # the mirror equals the device coordinates
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
        if self._x is None:
            self._host_x = np.zeros((0, self.dim))
        elif not self._host_valid or self._host_x is None or self._host_x.shape != tuple(self._x.shape):
            if self._host_x is None or self._host_x.shape != tuple(self._x.shape):
                self._host_x = _core.host_array(tuple(self._x.shape), np.float64)
            torch.from_numpy(self._host_x).copy_(self._x)
            self._host_valid = True
        view = self._host_x.view()   # the mirror itself stays writeable; views carry the flag
        view.flags.writeable = self._writable
        return view

    def fn_particle_found(self):
        """A boolean Function: True where one of this swarm's particles serves
        the point (P/swarm/_swarm.py:419-475)."""
        if not hasattr(self, "_fn_particle_found"):
            self._fn_particle_found = _fn._ParticleFound(self)
        return self._fn_particle_found

    def add_variable(self, dataType, count):
        v = SwarmVariable(self, dataType, count)
        self._variables.append(v)
        return v

    @property
    def variables(self):
        """The swarm variables added to this swarm."""
        return list(self._variables)

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
        self._host_valid = False
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
            self._x.copy_(torch.from_numpy(self._host_x))   # the mirror stays equal to the device copy
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
            v._set_rows(v._data[src])
        self._x, self._owner, self._off, self._lst = x, owner, off, lst
        self._host_valid = False

    # -- the PIC integration swarm ---------------------------------------------
    @property
    def _voronoi_swarm(self):
        if self._voronoi is None:
            self._voronoi = VoronoiIntegrationSwarm(self)
        return self._voronoi


class GaussIntegrationSwarm:
    """Integration points at the tensor Gauss-Legendre points of every element
    (P/swarm/_integration_swarm.py:155-200): particleCount points per axis,
    3 by default (5 on Q2 meshes), from 1 to 5.  Systems and integrals that
    take one integrate on those points."""

    def __init__(self, mesh, particleCount=None, **kwargs):
        if particleCount is None:
            particleCount = 5 if mesh.elementType.upper().startswith("Q2") else 3
        if not isinstance(particleCount, int) or isinstance(particleCount, bool):
            raise ValueError("'particleCount' parameter must be of type 'int'.")
        if particleCount not in (1, 2, 3, 4, 5):
            raise ValueError("'particleCount' must take a value in [1,5].")
        self.mesh = mesh
        self._particleCount = particleCount

    @property
    def particleCount(self):
        return self._particleCount

    @property
    def particleLocalCount(self):
        return self.mesh.elementsGlobal * self._particleCount ** self.mesh.dim


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


# ---------------------------------------------------------------------------
# Host-side layouts.  The reference generates these positions serially on the
# host at swarm set-up (no GPU counterpart is needed for a one-time fill); the
# arithmetic below follows its expressions so that positions are bit-identical.
# ---------------------------------------------------------------------------
_PM_M = 2147483647

# Sobol generators of the first three axes, from the reference's table
# (L/StgDomain/Utils/src/SobolGenerator.c:288-321, the initialisation of Joe and
# Kuo, ACM TOMS 29(1), 2003): polynomial degree, coefficient, initial direction
# numbers.
_SOBOL_TABLE = ((1, 0, (1,)), (2, 1, (1, 1)), (3, 1, (1, 3, 7)))
_SOBOL_BITS = 30   # WORDLENGTH of SobolGenerator_GetNextNumber


def _sobol_direction_numbers(axis):
    """Direction numbers v_0..v_29 of an axis' generator by the recurrence of
    SobolGenerator_GetDirectionalNumber (SobolGenerator.c:179-216)."""
    deg, coef, init = _SOBOL_TABLE[axis]
    v = list(init)
    while len(v) < _SOBOL_BITS:
        i = len(v)
        r = last = 0
        for c in range(deg):
            if c == deg - 1 or (coef >> (deg - 2 - c)) & 1:
                last = v[i - 1 - c]
                r ^= ((1 << (c + 1)) * last) & 0xFFFFFFFF
        v.append((r ^ last) & 0xFFFFFFFF)
    return v


def _sobol(axis, n):
    """The n-th value (n >= 1, uint64 array) that successive
    SobolGenerator_GetNextNumber calls return (SobolGenerator.c:218-241): the
    Gray code of n selects the direction numbers XOR-ed into the 30-bit word."""
    v = _sobol_direction_numbers(axis)
    g = n ^ (n >> np.uint64(1))
    word = np.zeros(n.shape, dtype=np.uint64)
    for b in range(_SOBOL_BITS):
        bit = (g >> np.uint64(b)) & np.uint64(1)
        word ^= bit * np.uint64(v[b] << (_SOBOL_BITS - b - 1))
    return word.astype(np.float64) / float(1 << _SOBOL_BITS)


def _pm_draws(state, n):
    """The next n states of the Park-Miller stream (Random.c:23-53) after
    `state`, by jump-ahead powers of 16807, and the state after the last."""
    if n == 0:
        return np.zeros(0, dtype=np.uint64), state
    M = np.uint64(_PM_M)
    pw = np.empty(n, dtype=np.uint64)       # pw[j] = 16807^(j+1) mod M
    pw[0] = 16807
    m = 1
    while m < n:
        k = min(m, n - m)
        pw[m:m + k] = (pw[:k] * pw[m - 1]) % M
        m += k
    st = (pw * np.uint64(state)) % M
    return st, int(st[-1])


def _shape_values(dim, order, xi):
    """Shape functions at local coordinates xi[n, dim], lexicographic nodes, in
    the expressions of BilinearElementType.c:179-211, TrilinearElementType.c:
    215-274, Biquadratic.c:138-200 and Triquadratic.c:193-300."""
    x = xi[:, 0]
    y = xi[:, 1]
    if dim == 2 and order == 1:
        return np.stack([0.25 * (1.0 - x) * (1.0 - y), 0.25 * (1.0 + x) * (1.0 - y),
                         0.25 * (1.0 - x) * (1.0 + y), 0.25 * (1.0 + x) * (1.0 + y)], 1)
    if dim == 3 and order == 1:
        z = xi[:, 2]
        out = []
        for c in range(2):
            fz = (1.0 - z) if c == 0 else (1.0 + z)
            for b in range(2):
                fy = (1.0 - y) if b == 0 else (1.0 + y)
                for a in range(2):
                    fx = (1.0 - x) if a == 0 else (1.0 + x)
                    out.append(0.125 * fx * fy * fz)
        return np.stack(out, 1)
    if dim == 2:
        a0, b0 = x - 1.0, y - 1.0
        a1, b1 = 1.0 - x * x, 1.0 - y * y
        a2, b2 = x + 1.0, y + 1.0
        m0, m1, m2 = 0.5 * x, 0.5 * y, 0.25 * x * y
        return np.stack([m2 * a0 * b0, m1 * a1 * b0, m2 * a2 * b0, m0 * a0 * b1, a1 * b1, m0 * a2 * b1,
                         m2 * a0 * b2, m1 * a1 * b2, m2 * a2 * b2], 1)
    z = xi[:, 2]
    A = (x - 1.0, 1.0 - x * x, x + 1.0)
    B = (y - 1.0, 1.0 - y * y, y + 1.0)
    C = (z - 1.0, 1.0 - z * z, z + 1.0)
    m0, m1, m2 = 0.5 * x, 0.5 * y, 0.5 * z
    m3, m4, m5 = 0.25 * x * y, 0.25 * x * z, 0.25 * y * z
    m6 = 0.125 * x * y * z
    mfull = (None, m2, m1, m5, m0, m4, m3, m6)   # by corner axes (x: 4, y: 2, z: 1)
    out = []
    for n in range(27):
        a, b, c = n % 3, (n // 3) % 3, n // 9
        sel = (a != 1) * 4 + (b != 1) * 2 + (c != 1)
        out.append(mfull[sel] * A[a] * B[b] * C[c] if sel else A[a] * B[b] * C[c])
    return np.stack(out, 1)


def _local_to_global(mesh, el, xi):
    """FeMesh_CoordLocalToGlobal (L/StgFEM/Discretisation/src/FeMesh.c:333-360):
    x = sum over the element's nodes, in order, of N_A(xi) times the vertex."""
    N = _shape_values(mesh.dim, mesh._order, xi)
    X = mesh.data
    en = mesh.data_elementNodes[el]
    out = np.zeros((len(el), mesh.dim))
    for a in range(N.shape[1]):
        va = X[en[:, a]]
        for d in range(mesh.dim):
            out[:, d] += N[:, a] * va[:, d]
    return out


def _space_filler_positions(mesh, ppc, state, chunk=1 << 22):
    """PerCellSpaceFillerLayout (L/StgFEM/Utils/src/MeshParticleLayout.c:194-230,
    filltype 0): cells in order, particles in order; one draw of the shared
    stream per particle, and when it exceeds 0.9 every axis' generator skips one
    value; local coordinate = (1 - -1) * sobol + -1.  Returns (x, state)."""
    n_el = mesh.elementsGlobal
    total = n_el * ppc
    out = np.empty((total, mesh.dim))
    skipped = 0
    for start in range(0, total, chunk):
        n = min(chunk, total - start)
        st, state = _pm_draws(state, n)
        rnd = (1.0 - 0.0) * st.astype(np.float64) / float(_PM_M) + 0.0
        skip = (rnd > 0.9).astype(np.uint64)
        idx = np.arange(start + 1, start + n + 1, dtype=np.uint64) + np.uint64(skipped) + np.cumsum(skip)
        skipped += int(skip.sum())
        xi = np.stack([(1.0 - -1.0) * _sobol(d, idx) + -1.0 for d in range(mesh.dim)], 1)
        out[start:start + n] = _local_to_global(mesh, np.arange(start, start + n) // ppc, xi)
    return out, state


def _gauss_positions(mesh, count):
    """PerCellGaussLayout (L/StgFEM/Discretisation/src/IrregularMeshGaussLayout.c:
    143-177): per cell count^dim particles at the Gauss-Legendre abscissae,
    x index fastest."""
    x1, _ = np.polynomial.legendre.leggauss(count)
    per = count ** mesh.dim
    p = np.arange(per)
    loc = [x1[p % count], x1[(p // count) % count]] + ([x1[p // (count * count)]] if mesh.dim == 3 else [])
    xi = np.tile(np.stack(loc, 1), (mesh.elementsGlobal, 1))
    el = np.repeat(np.arange(mesh.elementsGlobal), per)
    return _local_to_global(mesh, el, xi), per


def _set_per_cell(swarm, x, per):
    """Particles generated per cell in cell order: owner = generating cell."""
    ctx = swarm.mesh.ctx
    n_el = swarm.mesh.elementsGlobal
    dev = ctx.device
    xt = torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    owner = torch.arange(n_el, device=dev, dtype=torch.int32).repeat_interleave(per)
    off = (torch.arange(n_el + 1, device=dev, dtype=torch.int64) * per).to(torch.int32)
    lst = torch.arange(n_el * per, device=dev, dtype=torch.int32)
    swarm._set_particles(xt, owner, off, lst)


class PerCellSpaceFillerLayout(_ParticleLayoutAbstract):
    """Per-element quasi-random (Sobol) layout (P/swarm/layouts.py:146-184,
    L/StgFEM/Utils/src/MeshParticleLayout.c:194-230).  Constructing the layout
    seeds the process-wide stream with 13, as _MeshParticleLayout_Init does."""

    def __init__(self, swarm, particlesPerCell, **kwargs):
        if not isinstance(particlesPerCell, int):
            raise TypeError("'particlesPerCell' object passed in must be of type 'int'.")
        if particlesPerCell < 1:
            raise ValueError("'particlesPerCell' object passed in must take a value greater than zero.")
        super().__init__(swarm)
        self.particlesPerCell = particlesPerCell
        _RNG["state"] = _core.rng_seed(13)

    def _populate(self):
        x, _RNG["state"] = _space_filler_positions(self.swarm.mesh, self.particlesPerCell, _RNG["state"])
        _set_per_cell(self.swarm, x, self.particlesPerCell)


class PerCellGaussLayout(_ParticleLayoutAbstract):
    """Particles at the Gauss points of every element (P/swarm/layouts.py:53-108)."""

    def __init__(self, swarm, gaussPointCount, **kwargs):
        if not isinstance(gaussPointCount, int):
            raise TypeError("'gaussPointCount' object passed in must be of type 'int'")
        if gaussPointCount not in (1, 2, 3, 4, 5):
            raise ValueError("'gaussPointCount' object passed in must take a value between \n between 1 and 5 "
                             "inclusive.")
        super().__init__(swarm)
        self.gaussPointCount = gaussPointCount

    def _populate(self):
        x, per = _gauss_positions(self.swarm.mesh, self.gaussPointCount)
        _set_per_cell(self.swarm, x, per)


class layouts:
    PerCellRandomLayout = PerCellRandomLayout
    PerCellSpaceFillerLayout = PerCellSpaceFillerLayout
    PerCellGaussLayout = PerCellGaussLayout
