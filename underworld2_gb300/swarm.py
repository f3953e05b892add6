"""Particle swarms on the GPU (``uw.swarm`` subset).

The particle state -- coordinates, owning element and the per-element cell
tables -- lives on the device.  Particle index order never changes (no
particle deletion), so swarm variables are plain arrays indexed by particle.
Reference: P/swarm/_swarm.py, P/swarm/_swarmabstract.py, P/swarm/layouts.py,
P/swarm/_integration_swarm.py.
"""
import contextlib

import numpy as np
import torch

from . import _core
from . import function as _fn

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
        x = kept if self._x is None else torch.cat([self._x, kept])
        self._set_particles(x, rebuild=True)
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
        """Swarm_UpdateAllParticleOwners with the reference's escape check (P/swarm/_swarm.py:613-654)."""
        lost = self.mesh.ctx.update_owners(self._x, self._owner, self._off, self._lst)
        if lost and not self.particleEscape:
            raise RuntimeError("Particles appear to have left the domain, but swarm flag `particleEscape` is False. "
                               "Check your velocity field or your particle relocation routines, or set the "
                               "`particleEscape` swarm constructor parameter to True to allow escape.")
        self._host_x = None
        self._toggle_state()
        return lost

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
