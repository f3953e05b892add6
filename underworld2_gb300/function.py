"""The subset of ``underworld.function`` that the PIC Stokes path needs.

Functions are small expression trees evaluated once per integration point
into arrays (viscosity, body force, compressibility), on the device with
torch tensor arithmetic, mirroring the reference's per-point evaluation
(``SwarmVariableFn::getFunction`` maps an integration point to its material
particle, L/Underworld/Function/src/SwarmVariableFn.cpp:30-110; coordinate
inputs are the integration point's global position).

Supported: constants and tuples, ``input()``/``coord()``, swarm and mesh
variables and mesh-variable gradients, arithmetic (+ - * / **, unary -),
comparisons and logical and/or, the ``math`` functions of
P/function/math.py, ``misc.min/max``, ``tensor.symmetric/antisymmetric/
second_invariant/deviatoric`` (L/StgDomain/Geometry/src/TensorMath.c
conventions: full tensors row-major, symmetric tensors [00, 11, (22,) 01,
(02, 12)]), ``shape.Polygon``, ``branching.map/conditional``,
``view.min_max``, ``view.count``, ``exception.SafeMaths``, ``exception.CustomException``,
``rheology.stress_limiting_viscosity`` and the fixed-wall analytic solutions
``analytic.SolDB2d``/``SolDB3d``.  ``Function.evaluate`` accepts
coordinates, a mesh or a swarm, as the reference's.
"""
import math as _pymath
import numbers

import numpy as np
import torch


class EvalContext:
    """Where to evaluate: integration points with their particle ids and
    global coordinates (coords computed on demand).  ``swarm`` is set when the
    points are a swarm's own particles; ``map_swarm`` when they are integration
    points whose particle ids come from that swarm's integration-point map."""

    swarm = None
    map_swarm = None
    check_domain = False

    def __init__(self, particle_ids, coords_fn, device, lib_ctx=None, pid32=None):
        self.pid = particle_ids
        self._coords_fn = coords_fn
        self._coords = None
        self.device = device
        self.lib_ctx = lib_ctx     # the mesh's libuwg context: compiled evaluation (uwg_fn_eval)
        self.pid32 = pid32         # int32 particle id of each point

    @property
    def coords(self):
        if self._coords is None:
            self._coords = self._coords_fn()
        return self._coords

    @property
    def n(self):
        return self.pid.shape[0]


class Function:
    """Base class: ``_eval(ctx)`` returns a float64 tensor of shape (n, k).
    ``_kind`` is the value type where it matters: "tensor" (full, row-major),
    "symtensor" or None; ``_bool`` marks boolean results (stored as 0/1)."""

    _kind = None
    _bool = False
    _int = False      # integer results (integer constants): evaluate() returns int32

    @staticmethod
    def convert(obj):
        if obj is None or isinstance(obj, Function):
            return obj
        if isinstance(obj, numbers.Number):
            return constant(obj)
        if isinstance(obj, np.generic):
            return Function.convert(obj.item())
        if isinstance(obj, np.ndarray):
            return Function.convert(obj.tolist())
        if isinstance(obj, (tuple, list)):
            parts = [Function.convert(o) for o in obj]
            if all(isinstance(p, constant) and p._sig[1] == 1 for p in parts):
                tags = {p._sig[0] for p in parts}
                if len(tags) == 1:
                    return constant([p.value for p in parts])
                if "bool" not in tags:      # ints and floats together: a float vector
                    return constant([float(p.value) for p in parts])
            return _Vector(parts)
        if hasattr(obj, "_as_function"):
            return obj._as_function()
        try:
            return constant(obj)
        except ValueError as e:
            # the reference converts through misc.constant and re-raises its error
            # with this note prepended (P/function/_function.py:230-265)
            raise ValueError("An exception was raised while try to convert an object to an Underworld2 function. "
                             "Usually this occurs because you didn't pass in the correct object. Please check your "
                             "function arguments! Note that only python types 'int', 'float' or 'bool' (and "
                             "iterables of these types) are convertible to functions.\n\n" + str(e)) from None

    def _eval(self, ctx):
        raise NotImplementedError

    def evaluate_at(self, ctx):
        v = self._eval(ctx)
        if v.dim() == 1:
            v = v[:, None]
        if v.shape[0] == 1 and ctx.n != 1:
            v = v.expand(ctx.n, v.shape[1])
        return v

    def depends_on(self, kinds):
        return any(c.depends_on(kinds) for c in self._children())

    def _children(self):
        return []

    def evaluate(self, inputData=None, inputType=None):
        """Values at coordinates (float, tuple, list or [n, dim] array), at the
        nodes of a mesh or at the particles of a swarm (P/function/_function.py:808-930).
        Returns an [n, k] numpy array (bool for boolean functions)."""
        ctx = _input_context(inputData)
        dt = bool if self._bool else (np.int32 if self._int else np.float64)
        if ctx.n == 0:
            return np.zeros((0, 1), dtype=dt)
        v = self.evaluate_at(ctx).cpu().numpy()
        return v != 0 if self._bool else np.array(v, dtype=dt)

    def evaluate_global(self, inputData, inputType=None):
        """Values at global coordinates, points outside the domain skipped
        (P/function/_function.py:654-759).  One process holds the whole domain
        here, so this process is the root and gets the [n, k] result; rows of
        points that no evaluation found stay zero, and RuntimeError is raised
        when none was found.  Mesh, swarm and index-set inputs are refused."""
        from .container import ObjectifiedIndexSet
        if hasattr(inputData, "particleCoordinates") or hasattr(inputData, "_axes") or \
                isinstance(inputData, ObjectifiedIndexSet):
            raise TypeError("This 'inputData' type is not currently supported for global function evaluation.")
        if isinstance(inputData, np.ndarray):
            pts = inputData
        else:
            pts = np.atleast_2d(np.asarray(inputData if not isinstance(inputData, float) else (inputData,),
                                           dtype=np.float64))
        try:
            return self.evaluate(pts, inputType)
        except ValueError:
            pass                       # some point lies outside the domain: point by point
        out = None
        for i in range(len(pts)):
            try:
                v = self.evaluate(pts[i:i + 1], inputType)
            except ValueError:
                continue
            if out is None:
                out = np.zeros((len(pts), v.shape[1]), dtype=v.dtype)
            out[i] = v[0]
        if out is None:
            raise RuntimeError("No results were found anywhere in the domain for provided input.")
        return out

    def integrate(self, mesh):
        """Volume integral over the mesh (P/function/_function.py:775-800)."""
        from .utils import Integral
        return Integral(self, mesh).evaluate()

    # arithmetic
    def __add__(self, o): return _Bin(torch.add, self, Function.convert(o))
    def __radd__(self, o): return _Bin(torch.add, Function.convert(o), self)
    def __sub__(self, o): return _Bin(torch.sub, self, Function.convert(o))
    def __rsub__(self, o): return _Bin(torch.sub, Function.convert(o), self)
    def __mul__(self, o): return _Bin(torch.mul, self, Function.convert(o))
    def __rmul__(self, o): return _Bin(torch.mul, Function.convert(o), self)
    def __truediv__(self, o): return _Bin(torch.div, self, Function.convert(o))
    def __rtruediv__(self, o): return _Bin(torch.div, Function.convert(o), self)
    def __pow__(self, o): return _Bin(torch.pow, self, Function.convert(o))
    def __neg__(self): return _Un(torch.neg, self)
    def __lt__(self, o): return _Bool(lambda a, b: a < b, self, Function.convert(o), "lt")
    def __le__(self, o): return _Bool(lambda a, b: a <= b, self, Function.convert(o), "le")
    def __gt__(self, o): return _Bool(lambda a, b: a > b, self, Function.convert(o), "gt")
    def __ge__(self, o): return _Bool(lambda a, b: a >= b, self, Function.convert(o), "ge")
    def __and__(self, o): return _Bool(lambda a, b: (a != 0) & (b != 0), self, Function.convert(o), "and")
    def __or__(self, o): return _Bool(lambda a, b: (a != 0) | (b != 0), self, Function.convert(o), "or")
    def __xor__(self, o): return _Bool(lambda a, b: (a != 0) ^ (b != 0), self, Function.convert(o), "xor")

    def __getitem__(self, i):
        return _Index(self, i)


def _const_tag(v):
    if isinstance(v, (bool, np.bool_)):
        return "bool"
    if isinstance(v, numbers.Integral):
        return "int"
    if isinstance(v, numbers.Real):
        return "double"
    return None


def _const_signature(value):
    """(type, size) of a constant's value: a bool, int or float, or a non-empty
    iterable of one of those types (P/function/misc.py:73-126)."""
    tag = _const_tag(value)
    if tag is not None:
        return tag, 1
    try:
        items = tuple(iter(value))
    except TypeError:
        raise ValueError("'value' object provided to Constant Function constructor does not appear to be valid. "
                         "Only python types 'int', 'float' and 'bool' are acceptable, or iterable objects "
                         "homogeneous in these types. Provided object was of type '{}'."
                         .format(type(value).__name__))
    if not items:
        raise ValueError("'value' object provided to Constant function appears to be an iterable, but seems to be "
                         "of zero size. Iterable values must be of non-zero size.")
    tag = _const_tag(items[0])
    if tag is None:
        raise ValueError("'value' object provided to Constant function appears to be an iterable, but does not "
                         "appear to contain objects of python type 'int', 'float' or 'bool'.")
    if any(_const_tag(v) != tag for v in items[1:]):
        raise ValueError("'value' object provided to Constant function appears to be an iterable, but does not "
                         "appear to be homogeneous in type. Objects in iterable must all be of python type 'int', "
                         "'float' or 'bool'.")
    return tag, len(items)


class constant(Function):
    """A constant value (P/function/misc.py:13-126).  The value keeps its type:
    bools evaluate to bool, ints to int32, floats to float64; `value` may be
    reset to another value of the same type and size."""

    def __init__(self, value):
        self._sig = _const_signature(value)
        self._value = value
        self._bool = self._sig[0] == "bool"
        self._int = self._sig[0] == "int"

    @property
    def value(self):
        return self._value

    @value.setter
    def value(self, value):
        tag, size = _const_signature(value)
        if tag != self._sig[0]:
            raise TypeError("'value' object passed in must be of identical type to that used in construction of "
                            "this function.")
        if size != self._sig[1]:
            raise TypeError("'value' object passed in must be of identical size to that used in construction of "
                            "this function.")
        self._value = value

    def _eval(self, ctx):
        t = torch.as_tensor(self.value, dtype=torch.float64, device=ctx.device)
        return t.reshape(1, -1)

    def depends_on(self, kinds):
        return False


class _Vector(Function):
    def __init__(self, parts):
        self.parts = parts

    def _children(self):
        return self.parts

    def _eval(self, ctx):
        cols = [p.evaluate_at(ctx) for p in self.parts]
        return torch.cat(cols, dim=1)


class _Bin(Function):
    def __init__(self, op, a, b):
        self.op, self.a, self.b = op, a, b
        # a scalar times (or plus) a tensor keeps the tensor's type
        self._kind = a._kind or b._kind

    def _children(self):
        return [self.a, self.b]

    def _eval(self, ctx):
        return self.op(self.a.evaluate_at(ctx), self.b.evaluate_at(ctx))


class _Bool(Function):
    _bool = True

    def __init__(self, op, a, b, name=None):
        self.op, self.a, self.b, self.name = op, a, b, name

    def _children(self):
        return [self.a, self.b]

    def _eval(self, ctx):
        return self.op(self.a.evaluate_at(ctx), self.b.evaluate_at(ctx)).double()


class _Un(Function):
    def __init__(self, op, a):
        self.op, self.a = op, a
        self._kind = a._kind

    def _children(self):
        return [self.a]

    def _eval(self, ctx):
        return self.op(self.a.evaluate_at(ctx))


class _Index(Function):
    def __init__(self, a, i):
        self.a, self.i = a, i

    def _children(self):
        return [self.a]

    def _eval(self, ctx):
        return self.a.evaluate_at(ctx)[:, self.i: self.i + 1]


class input(Function):
    """The global coordinate of the evaluation point."""

    def _eval(self, ctx):
        return ctx.coords

    def depends_on(self, kinds):
        return "coord" in kinds


coord = input


class _SwarmVar(Function):
    def __init__(self, var):
        self.var = var
        # integer swarm variables evaluate to integers (the reference's IO_int output)
        self._int = getattr(var, "dataType", "double") in ("int", "char", "short", "long")

    def _check_swarm(self, ctx):
        other = getattr(ctx, "swarm", None)
        if other is not None and other is not self.var.swarm:
            raise ValueError("'ParticleCoordinate' input and `SwarmVariableFn` function appear to be based on "
                             "different swarms.")

    def _eval(self, ctx):
        self._check_swarm(ctx)
        d = self.var._device_data()
        if d.dim() == 1:
            d = d[:, None]
        pid = ctx.pid.long()
        if pid.numel() and bool((pid < 0).any()):
            pid = _closest_particles(self.var.swarm, ctx.coords, pid)
        return d[pid].double()

    def evaluate(self, inputData=None, inputType=None):
        """The variable's own values, in its own type (the reference's IO_char ...
        IO_double outputs): at a swarm's particles, or the nearest particle's at
        coordinates or a mesh's nodes."""
        ctx = _input_context(inputData)
        self._check_swarm(ctx)
        data = self.var._data
        if ctx.n == 0:
            return np.zeros((0, data.shape[1]), dtype=data.dtype)
        pid = ctx.pid.long()
        if bool((pid < 0).any()):
            pid = _closest_particles(self.var.swarm, ctx.coords, pid)
        return np.array(data[pid.cpu().numpy()])

    def depends_on(self, kinds):
        return "swarm" in kinds


def _closest_particles(swarm, pts, pid, chunk_elems=1 << 24):
    """Index of the closest particle of `swarm` to each point that has none yet
    (pid < 0): a swarm variable evaluated at plain coordinates takes its nearest
    particle's value (SwarmVariableFn, L/Underworld/Function/src/SwarmVariableFn.cpp:
    129-171, over GeneralSwarm_GetClosestParticles).  Exhaustive search in chunks;
    ties go to the lowest particle index."""
    if pts.shape[1] != swarm.dim:
        raise RuntimeError("Function input dimensionality (%d) does not appear to match swarm variable "
                           "dimensionality (%d)." % (pts.shape[1], swarm.dim))
    x = swarm._x
    if x is None or x.shape[0] == 0:
        raise RuntimeError("Unable to evaluate SwarmVariable: the swarm holds no particles.")
    x = x.to(device=pts.device, dtype=torch.float64)
    pid = pid.clone()
    todo = torch.nonzero(pid < 0).flatten()
    step = max(1, chunk_elems // x.shape[0])
    for s in range(0, todo.numel(), step):
        idx = todo[s:s + step]
        q = pts[idx].to(torch.float64)
        d2 = ((q[:, None, :] - x[None, :, :]) ** 2).sum(-1)
        pid[idx] = torch.argmin(d2, dim=1)
    return pid


class _ParticleFound(Function):
    """True where a particle of `swarm` serves the point (ParticleFound,
    L/Underworld/Function/src/ParticleFound.cpp:26-95): at the swarm's own
    particles; at integration points, when the point's element holds one of the
    swarm's particles (the point's particle map found one); False at plain
    coordinates."""
    _bool = True

    def __init__(self, swarm):
        self.swarm = swarm

    def _eval(self, ctx):
        n = ctx.n
        if getattr(ctx, "swarm", None) is not None:
            v = torch.full((n, 1), 1.0 if ctx.swarm is self.swarm else 0.0, dtype=torch.float64, device=ctx.device)
        elif getattr(ctx, "map_swarm", None) is self.swarm:
            v = (ctx.pid >= 0).to(torch.float64)[:, None]
        else:
            v = torch.zeros((n, 1), dtype=torch.float64, device=ctx.device)
        return v

    def depends_on(self, kinds):
        return "swarm" in kinds


def _check_in_domain(var, ctx):
    """At user-given coordinates, a mesh variable is defined only inside its
    mesh: the reference raises for a point outside (FeVariableFn.cpp:82-92)."""
    if not getattr(ctx, "check_domain", False):
        return
    m = var._primary()
    x = ctx.coords
    if x.shape[1] != m.dim:
        return
    lo = torch.tensor(m.minCoord, dtype=x.dtype, device=x.device)
    hi = torch.tensor(m.maxCoord, dtype=x.dtype, device=x.device)
    bad = ((x < lo) | (x > hi)).any(1)
    if bool(bad.any()):
        p = x[int(bad.nonzero()[0, 0])].tolist()
        raise ValueError("FeVariable interpolation at location (%s) does not appear to be valid.\n"
                         "Location is probably outside local domain." % ", ".join("%g" % v for v in p))


class _MeshVar(Function):
    def __init__(self, var):
        self.var = var

    def _eval(self, ctx):
        _check_in_domain(self.var, ctx)
        return self.var._interpolate(ctx.coords)

    def depends_on(self, kinds):
        return "coord" in kinds or "mesh" in kinds


def _unary(op):
    return staticmethod(lambda fn=None: _Un(op, Function.convert(fn) if fn is not None else input()))


class _MeshGrad(Function):
    def __init__(self, var):
        self.var = var
        self._kind = "tensor" if var.nodeDofCount > 1 else None

    def _eval(self, ctx):
        _check_in_domain(self.var, ctx)
        return self.var._interpolate_grad(ctx.coords)

    def depends_on(self, kinds):
        return "coord" in kinds or "mesh" in kinds


class math:
    """Elementwise functions of P/function/math.py (the argument defaults to input())."""
    cos = _unary(torch.cos)
    sin = _unary(torch.sin)
    tan = _unary(torch.tan)
    acos = _unary(torch.acos)
    asin = _unary(torch.asin)
    atan = _unary(torch.atan)
    cosh = _unary(torch.cosh)
    sinh = _unary(torch.sinh)
    tanh = _unary(torch.tanh)
    acosh = _unary(torch.acosh)
    asinh = _unary(torch.asinh)
    atanh = _unary(torch.atanh)
    exp = _unary(torch.exp)
    log = _unary(torch.log)
    log2 = _unary(torch.log2)
    log10 = _unary(torch.log10)
    sqrt = _unary(torch.sqrt)
    erf = _unary(torch.erf)
    erfc = _unary(torch.erfc)
    abs = _unary(torch.abs)

    @staticmethod
    def pow(fn1, fn2): return _Bin(torch.pow, Function.convert(fn1), Function.convert(fn2))

    @staticmethod
    def dot(fn1, fn2):
        f = _Bin(lambda x, y: (x * y).sum(dim=1, keepdim=True), Function.convert(fn1), Function.convert(fn2))
        f.name = "dot"
        return f


class _Map(Function):
    """branching.map (P/function/branching.py:102-140): keys are unsigned ints."""

    def __init__(self, fn_key, mapping, fn_default=None):
        if not mapping:
            raise ValueError("You must specify a mapping via the 'mapping' parameter.")
        if not isinstance(mapping, dict):
            raise TypeError("'mapping' object passed in must be of python type 'dict'")
        if fn_key is None:
            raise ValueError("You must specify a key function via the 'fn_key' parameter.")
        self.key = Function.convert(fn_key)
        self.mapping = {}
        for k, v in mapping.items():
            if not isinstance(k, numbers.Integral) or isinstance(k, bool) or k < 0:
                raise ValueError("Key '{}' not valid. Mapping keys must be unsigned integers.".format(k))
            f = Function.convert(v)
            if f is None:
                raise ValueError("'None' is not valid for mapped functions.")
            self.mapping[int(k)] = f
        self.default = Function.convert(fn_default)

    def _children(self):
        out = [self.key] + list(self.mapping.values())
        return out + ([self.default] if self.default is not None else [])

    def _eval(self, ctx):
        key = self.key.evaluate_at(ctx)[:, 0].round().long()
        out = None
        hit = torch.zeros(ctx.n, dtype=torch.bool, device=ctx.device)
        for k, f in self.mapping.items():
            v = f.evaluate_at(ctx)
            if out is None:
                out = torch.zeros((ctx.n, v.shape[1]), dtype=torch.float64, device=ctx.device)
            sel = key == k
            out[sel] = v.expand(ctx.n, v.shape[1])[sel]
            hit |= sel
        if self.default is not None:
            v = self.default.evaluate_at(ctx)
            out[~hit] = v.expand(ctx.n, v.shape[1])[~hit]
        elif not bool(hit.all()):
            k = int(key[~hit][0])
            raise RuntimeError("Error evaluating 'map' function.\nKey function evaluates to key (%d) which\n"
                               "does not appear to map to any functions, and no default function has been set." % k)
        return out


_NO_CLAUSE = ("Reached end of conditional statement. At least one of the clause conditions must evaluate to "
              "'True'.")
_NO_KEY = ("Error evaluating 'map' function.\nKey function evaluates to a key which\n"
           "does not appear to map to any functions, and no default function has been set.")


class _Conditional(Function):
    """branching.conditional (P/function/branching.py:143-230): the first clause
    whose condition holds gives the value."""

    def __init__(self, clauses):
        if not isinstance(clauses, (list, tuple)):
            raise TypeError("'clauses' object passed in must be of python type 'list' or 'tuple'")
        self.clauses = []
        for clause in clauses:
            if not isinstance(clause, (list, tuple)):
                raise TypeError("Clauses within the clause list must be of python type 'list' or 'tuple'")
            if len(clause) != 2:
                raise ValueError("Clauses tuples must be of length 2.")
            self.clauses.append((Function.convert(clause[0]), Function.convert(clause[1])))

    def _children(self):
        return [f for cv in self.clauses for f in cv]

    def _eval(self, ctx):
        out = None
        done = torch.zeros(ctx.n, dtype=torch.bool, device=ctx.device)
        for c, f in self.clauses:
            cond = c.evaluate_at(ctx)[:, 0] != 0
            v = f.evaluate_at(ctx)
            if out is None:
                out = torch.zeros((ctx.n, v.shape[1]), dtype=torch.float64, device=ctx.device)
            sel = cond & ~done
            out[sel] = v.expand(ctx.n, v.shape[1])[sel]
            done |= sel
        if not bool(done.all()):
            raise RuntimeError(_NO_CLAUSE)
        return out


class branching:
    @staticmethod
    def map(fn_key=None, mapping=None, fn_default=None, keyFunc=None, mappingDict=None):
        return _Map(fn_key if fn_key is not None else keyFunc, mapping if mapping is not None else mappingDict,
                    fn_default)

    @staticmethod
    def conditional(clauses):
        return _Conditional(clauses)


class misc:
    constant = constant

    @staticmethod
    def max(fn1, fn2):
        """Elementwise maximum of two scalar functions (P/function/misc.py)."""
        return _Bin(torch.maximum, Function.convert(fn1), Function.convert(fn2))

    @staticmethod
    def min(fn1, fn2):
        """Elementwise minimum of two scalar functions (P/function/misc.py)."""
        return _Bin(torch.minimum, Function.convert(fn1), Function.convert(fn2))


def _dim_of(k, kind):
    return {("tensor", 4): 2, ("tensor", 9): 3, ("symtensor", 3): 2, ("symtensor", 6): 3}.get((kind, k))


class _TensorFn(Function):
    def __init__(self, what, fn):
        self.what, self.a = what, Function.convert(fn)
        need = {"symmetric": "tensor", "antisymmetric": "tensor", "deviatoric": "symtensor"}.get(what)
        if need and self.a._kind != need:
            raise ValueError("TensorFunc expects %s input for '%s'" % ("Tensor" if need == "tensor" else
                                                                      "SymmetricTensor", what))
        if what == "second_invariant" and self.a._kind not in ("tensor", "symtensor"):
            raise ValueError("second_invariant expects a Tensor or SymmetricTensor input")
        self._kind = {"symmetric": "symtensor", "antisymmetric": "tensor", "deviatoric": "symtensor"}.get(what)

    def _children(self):
        return [self.a]

    def _eval(self, ctx):
        t = self.a.evaluate_at(ctx)
        dim = _dim_of(t.shape[1], self.a._kind)
        if dim is None:
            raise ValueError("tensor function input has %d components" % t.shape[1])
        if self.a._kind == "tensor":
            F = t.reshape(-1, dim, dim)
            if self.what == "symmetric":      # TensorArray_GetSymmetricPart (TensorMath.c:229-270)
                S = 0.5 * (F + F.transpose(1, 2))
                cols = [F[:, 0, 0], F[:, 1, 1]] + ([F[:, 2, 2]] if dim == 3 else []) + [S[:, 0, 1]] + \
                    ([S[:, 0, 2], S[:, 1, 2]] if dim == 3 else [])
                return torch.stack(cols, dim=1)
            if self.what == "antisymmetric":  # TensorArray_GetAntisymmetricPart (:167-227)
                return (0.5 * (F - F.transpose(1, 2))).reshape(-1, dim * dim)
            return torch.sqrt(0.5 * (t * t).sum(dim=1, keepdim=True))   # TensorArray_2ndInvariant (:379-405)
        # symmetric storage
        diag = t[:, :dim]
        off = t[:, dim:]
        if self.what == "second_invariant":   # SymmetricTensor_2ndInvariant (:409-437)
            return torch.sqrt(0.5 * (diag * diag).sum(dim=1, keepdim=True) + (off * off).sum(dim=1, keepdim=True))
        mean = diag.sum(dim=1, keepdim=True) / dim      # deviatoric (Tensor.cpp get_deviatoric)
        return torch.cat([diag - mean, off], dim=1)


class tensor:
    """Tensor functions of P/function/tensor.py."""

    @staticmethod
    def symmetric(fn): return _TensorFn("symmetric", fn)

    @staticmethod
    def antisymmetric(fn): return _TensorFn("antisymmetric", fn)

    @staticmethod
    def second_invariant(fn): return _TensorFn("second_invariant", fn)

    @staticmethod
    def deviatoric(fn): return _TensorFn("deviatoric", fn)


class _Polygon(Function):
    """Inside test of _PolygonShape_IsCoordInside (L/StgDomain/Shape/src/PolygonShape.c:268-316):
    the signed angles subtended by the edges sum to +-2 pi inside, 0 outside."""
    _bool = True

    def __init__(self, vertices, fn=None):
        if not isinstance(vertices, np.ndarray):
            raise TypeError("Provided 'vertices' must be a numpy array.")
        if len(vertices.shape) != 2:
            raise TypeError("Provided 'vertices' array must be 2 dimensional.")
        if vertices.shape[0] < 3:
            raise TypeError("Provided 'vertices' array must contain at least 3 vertices.")
        if vertices.shape[1] != 2:
            raise TypeError("Provided 'vertices' array must contain 2d vectors.")
        self.v = np.array(vertices, dtype=np.float64)
        self.a = Function.convert(fn) if fn is not None else input()

    def _children(self):
        return [self.a]

    def _eval(self, ctx):
        p = self.a.evaluate_at(ctx)
        if p.shape[1] not in (2, 3):
            raise ValueError("Polygon shape expects input to be be 2 or 3 dimensional vector.")
        x, y = p[:, 0], p[:, 1]
        V = torch.from_numpy(self.v).to(p.device)
        total = torch.zeros_like(x)
        for i in range(len(self.v)):
            sx, sy = x - V[i, 0], y - V[i, 1]
            j = (i + 1) % len(self.v)
            ex, ey = x - V[j, 0], y - V[j, 1]
            val = (sx * ex + sy * ey) / (torch.sqrt(sx * sx + sy * sy) * torch.sqrt(ex * ex + ey * ey))
            ang = torch.where(val >= 1.0, torch.zeros_like(val),
                              torch.where(val <= -1.0, torch.full_like(val, _pymath.pi), torch.acos(val)))
            cross = ex * sy - ey * sx
            total = torch.where(cross > 0.0, total + ang, total - ang)
        return (~(torch.abs(total) < _pymath.pi)).double()[:, None]


class shape:
    @staticmethod
    def Polygon(vertices, fn=None, *args, **kwargs): return _Polygon(vertices, fn)


class _SafeMaths(Function):
    def __init__(self, fn):
        self.a = Function.convert(fn)
        if not isinstance(self.a, Function):
            raise ValueError("provided 'fn' must a 'Function' or convertible.")
        self._kind = self.a._kind

    def _children(self):
        return [self.a]

    def _eval(self, ctx):
        v = self.a.evaluate_at(ctx)
        if not bool(torch.isfinite(v).all()):
            raise RuntimeError("Function evaluation produced a non-finite value (SafeMaths).")
        return v


class _CustomException(Function):
    """Pass-through of fn_input where fn_condition holds at every point; else a
    RuntimeError carrying fn_print's values at the first failing point
    (P/function/exception.py:69-140)."""

    def __init__(self, fn_input, fn_condition, fn_print=None):
        self.a = Function.convert(fn_input)
        self.cond = Function.convert(fn_condition)
        self.pr = Function.convert(fn_print) if fn_print is not None else None
        if not isinstance(self.a, Function) or not isinstance(self.cond, Function):
            raise ValueError("provided 'fn_input' and 'fn_condition' must be 'Function' or convertible.")
        self._kind = self.a._kind

    def _children(self):
        return [self.a, self.cond] + ([self.pr] if self.pr is not None else [])

    def _eval(self, ctx):
        ok = self.cond.evaluate_at(ctx)[:, 0] != 0
        if not bool(ok.all()):
            msg = "CustomException condition function has evaluated to False for current input!"
            if self.pr is not None:
                bad = int(torch.nonzero(~ok)[0])
                vals = self.pr.evaluate_at(ctx)[bad].to(torch.float64).tolist()
                msg += ("\nPrint function returns the following values (cast to double precision):\n    ( %s )"
                        % " ".join("%g" % v for v in vals))
            raise RuntimeError(msg)
        return self.a.evaluate_at(ctx)


class exception:
    @staticmethod
    def SafeMaths(fn, *args, **kwargs): return _SafeMaths(fn)

    @staticmethod
    def CustomException(fn_input, fn_condition, fn_print=None, *args, **kwargs):
        return _CustomException(fn_input, fn_condition, fn_print)


class _StressLimit(Function):
    def __init__(self, fn_stress, fn_stresslimit, fn_inputviscosity):
        self.s, self.lim, self.eta = (Function.convert(f) for f in (fn_stress, fn_stresslimit, fn_inputviscosity))
        for f, name in ((self.s, "fn_stress"), (self.lim, "fn_stresslimit"), (self.eta, "fn_inputviscosity")):
            if not isinstance(f, Function):
                raise ValueError("Provided '%s' must a 'Function' or convertible type." % name)

    def _children(self):
        return [self.s, self.lim, self.eta]

    def _eval(self, ctx):
        sII = _TensorFn("second_invariant", self.s).evaluate_at(ctx)
        lim = self.lim.evaluate_at(ctx)
        eta = self.eta.evaluate_at(ctx)
        return torch.where(sII > lim, eta * lim / sII, eta)


class rheology:
    @staticmethod
    def stress_limiting_viscosity(fn_stress, fn_stresslimit, fn_inputviscosity, *args, **kwargs):
        """eta * limit / stress_II where the stress invariant exceeds the limit
        (P/function/rheology.py; StressLimitingViscosity.cpp)."""
        return _StressLimit(fn_stress, fn_stresslimit, fn_inputviscosity)


class _MinMax(Function):
    """Pass-through that records the extremes of its (scalar) function, or of
    ``fn_norm`` for a non-scalar one, and the value of ``fn_auxiliary`` where they
    occur (P/function/view.py:16-245): the first point that strictly improves
    the record wins."""

    def __init__(self, fn, fn_norm=None, fn_auxiliary=None):
        self.a = Function.convert(fn)
        self.norm = Function.convert(fn_norm) if fn_norm is not None else None
        self.aux = Function.convert(fn_auxiliary) if fn_auxiliary is not None else None
        self.reset()

    def _children(self):
        return [self.a] + [f for f in (self.norm, self.aux) if f is not None]

    def reset(self):
        self._min, self._max = float("inf"), float("-inf")
        self._min_aux = self._max_aux = None

    def _eval(self, ctx):
        v = self.a.evaluate_at(ctx)
        if self.norm is not None:
            q = self.norm.evaluate_at(ctx)
            if q.shape[1] != 1:
                raise RuntimeError("Norm function does not return scalar results.")
        else:
            if v.shape[1] != 1:
                raise RuntimeError("Argument function does not return scalar results. You must also provide a "
                                   "function which calculates the required norm like quantity via the `fn_norm` "
                                   "parameter.")
            q = v
        if q.shape[0]:
            qv = q[:, 0]
            i_min, i_max = int(torch.argmin(qv)), int(torch.argmax(qv))
            lo, hi = float(qv[i_min]), float(qv[i_max])
            aux = self.aux.evaluate_at(ctx) if self.aux is not None else None
            if lo < self._min:
                self._min = lo
                if aux is not None:
                    self._min_aux = aux[i_min:i_min + 1].cpu().numpy().copy()
            if hi > self._max:
                self._max = hi
                if aux is not None:
                    self._max_aux = aux[i_max:i_max + 1].cpu().numpy().copy()
        return v

    def min_local(self): return self._min
    def max_local(self): return self._max
    def min_global(self): return self._min
    def max_global(self): return self._max

    def min_local_auxiliary(self): return self._min_aux
    def max_local_auxiliary(self): return self._max_aux
    def min_global_auxiliary(self): return self._min_aux
    def max_global_auxiliary(self): return self._max_aux


class _Count(Function):
    """Pass-through that counts its evaluations, one per point
    (P/function/view.py:385-440)."""

    def __init__(self, fn):
        self.a = Function.convert(fn)
        if not isinstance(self.a, Function):
            raise ValueError("provided 'fn' must a 'Function' or convertible.")
        self._kind = self.a._kind
        self._n = 0

    def _children(self):
        return [self.a]

    def _eval(self, ctx):
        v = self.a.evaluate_at(ctx)
        self._n += int(ctx.n)
        return v

    def count(self):
        return self._n

    def reset(self):
        self._n = 0


class view:
    @staticmethod
    def min_max(fn, fn_norm=None, fn_auxiliary=None, *args, **kwargs):
        """Pass-through that records the extrema of its input (of fn_norm where
        given, of the magnitude for vectors) over every evaluation (P/function/view.py)."""
        return _MinMax(fn, fn_norm, fn_auxiliary)

    @staticmethod
    def count(fn):
        """Pass-through that counts its evaluations (one per point)."""
        return _Count(fn)


# ---------------------------------------------------------------------------
# Analytic Stokes solutions with fixed velocity on every wall (P/function/analytic.py:568-656)
# ---------------------------------------------------------------------------
class _SolBase:
    """Base of the analytic solutions: fn_velocity, fn_pressure, fn_stress,
    fn_strainRate, fn_viscosity, fn_bodyforce, dim and nonlinear
    (P/function/analytic.py:62-79)."""
    eqn_bodyforce = None
    eqn_viscosity = None
    nonlinear = False


class _SolFixedBc(_SolBase):
    """Fields of an analytic solution as function graphs of the coordinates:
    fn_velocity, fn_pressure, fn_strainRate (symmetric-tensor order xx, yy[, zz], xy
    [, xz, yz]), fn_stress (2 eta strain rate), fn_viscosity and fn_bodyforce, the
    body force of -div(2 eta strain rate) + grad p = f."""

    fixed_walls = True

    def _finish(self, eta, vel, p, e, div_e, grad_p, grad_eta):
        """e: strain-rate components (matrix form, list of rows); div_e: the row
        divergences of e; grad_eta: the viscosity gradient (None when constant)."""
        d = self.dim
        self.fn_velocity = Function.convert(tuple(vel))
        self.fn_pressure = p
        sym = [e[0][0], e[1][1]] + ([e[2][2]] if d == 3 else []) + [e[0][1]] + ([e[0][2], e[1][2]] if d == 3 else [])
        self.fn_strainRate = Function.convert(tuple(sym))
        self.fn_viscosity = eta
        self.fn_stress = Function.convert(tuple(2.0 * eta * c for c in sym))
        force = []
        for i in range(d):
            f = -2.0 * eta * div_e[i] + grad_p[i]
            if grad_eta is not None:
                for j in range(d):
                    f = f - 2.0 * grad_eta[j] * e[i][j]
            force.append(f)
        self.fn_bodyforce = Function.convert(tuple(force))

    def get_bcs(self, velVar):
        """Velocity fixed on every wall at the analytic values, each wall's normal
        component shifted by the difference between its numerical and analytic
        fluxes (P/function/analytic.py:569-618).  The numerical flux is the exact
        integral of the nodal interpolant, sum_A w_A v_A with the tensor-product
        node weights of the wall (trapezoid on Q1, Simpson on Q2).  Returns the
        DirichletCondition."""
        from . import conditions as _cond
        from . import utils as _utils
        mesh = velVar.mesh
        ss = mesh.specialSets
        walls = ss["AllWalls_VertexSet"]
        velVar.data[walls.data] = self.fn_velocity.evaluate(mesh.data[walls.data])
        for ax, name in enumerate("IJK"[: self.dim]):
            for side in ("Min", "Max"):
                verts = ss["%s%s_VertexSet" % (side, name)]
                idx = verts.data
                num = float(np.dot(_wall_weights(mesh, idx, ax), velVar.data[idx, ax]))
                ana = _utils.Integral(self.fn_velocity[ax], mesh, integrationType="surface",
                                      surfaceIndexSet=verts).evaluate()
                velVar.data[idx, ax] -= num - float(np.asarray(ana).ravel()[0])
        return _cond.DirichletCondition(velVar, tuple(walls for _ in range(self.dim)))


def _node_weights_1d(c, order):
    """int N_i over an axis with node coordinates c: trapezoid (order 1), Simpson (order 2)."""
    w = np.zeros(len(c))
    for e in range((len(c) - 1) // order):
        a, b = e * order, (e + 1) * order
        h = c[b] - c[a]
        if order == 1:
            w[a] += 0.5 * h
            w[b] += 0.5 * h
        else:
            w[a] += h / 6.0
            w[a + 1] += 4.0 * h / 6.0
            w[b] += h / 6.0
    return w


def _wall_weights(mesh, idx, ax):
    """int N_A over the wall normal to axis ax for the wall's nodes idx."""
    axes = [np.asarray(a) for a in mesh._axes]
    nn = [len(a) for a in axes]
    w = np.ones(len(idx))
    rest = np.asarray(idx, dtype=np.int64)
    for d in range(len(axes)):
        i_d = rest % nn[d]
        rest = rest // nn[d]
        if d != ax:
            w *= _node_weights_1d(axes[d], mesh._order)[i_d]
    return w


class analytic:
    """The reference's analytic Stokes solutions (P/function/analytic.py): the
    fixed-wall SolDB2d and SolDB3d here, and the free-slip solutions SolA, SolB,
    SolC, SolCx, SolDA, SolH, SolKx, SolKz, SolM and the power-law SolNL
    (module _analytic_series)."""
    _SolBase = _SolBase

    class SolDB2d(_SolFixedBc):
        """Dohrmann & Bochev (Int. J. Numer. Meth. Fluids 46, 183-201, 2004), 2D, on the
        unit square: viscosity 1,
        u = (x + x^2 - 2xz + x^3 - 3xz^2 + x^2 z,  -z - 2xz + z^2 - 3x^2 z + z^3 - xz^2),
        p = xz + x + z + x^3 z^2 - 4/3 (z the second coordinate)."""
        eqn_viscosity = "1"

        def __init__(self, *args, **kwargs):
            self.dim = 2
            x, z = input()[0], input()[1]
            ux = x + x * x - 2.0 * x * z + x * x * x - 3.0 * x * z * z + x * x * z
            uz = -z - 2.0 * x * z + z * z - 3.0 * x * x * z + z * z * z - x * z * z
            p = x * z + x + z + x * x * x * z * z - 4.0 / 3.0
            exx = 1.0 + 2.0 * x - 2.0 * z + 3.0 * x * x - 3.0 * z * z + 2.0 * x * z
            exz = -x - z - 6.0 * x * z + 0.5 * x * x - 0.5 * z * z
            e = [[exx, exz], [exz, -exx]]
            div_e = [1.0 + z, 1.0 - x]
            grad_p = [z + 1.0 + 3.0 * x * x * z * z, x + 1.0 + 2.0 * x * x * x * z]
            self._finish(constant(1.0), [ux, uz], p, e, div_e, grad_p, None)

    class SolDB3d(_SolFixedBc):
        """Dohrmann & Bochev (2004), 3D, on the unit cube: viscosity
        eta = exp(1 - Beta (x(1-x) + y(1-y) + z(1-z))),
        u = (x + x^2 + xy + x^3 y,  y + xy + y^2 + x^2 y^2,  -2z - 3xz - 3yz - 5x^2 yz),
        p = xyz + x^2 y^3 z - 5/32."""

        def __init__(self, Beta=4., *args, **kwargs):
            self.dim = 3
            self.Beta = float(Beta)
            x, y, z = input()[0], input()[1], input()[2]
            b = self.Beta
            eta = math.exp(1.0 - b * (x * (1.0 - x) + y * (1.0 - y) + z * (1.0 - z)))
            u = [x + x * x + x * y + x * x * x * y,
                 y + x * y + y * y + x * x * y * y,
                 -2.0 * z - 3.0 * x * z - 3.0 * y * z - 5.0 * x * x * y * z]
            p = x * y * z + x * x * y * y * y * z - 5.0 / 32.0
            exx = 1.0 + 2.0 * x + y + 3.0 * x * x * y
            eyy = 1.0 + x + 2.0 * y + 2.0 * x * x * y
            ezz = -2.0 - 3.0 * x - 3.0 * y - 5.0 * x * x * y
            exy = 0.5 * x + 0.5 * x * x * x + 0.5 * y + x * y * y
            exz = -1.5 * z - 5.0 * x * y * z
            eyz = -1.5 * z - 2.5 * x * x * z
            e = [[exx, exy, exz], [exy, eyy, eyz], [exz, eyz, ezz]]
            div_e = [1.0 + 3.0 * x * y, 1.0 + x * x + y * y, -5.0 * y * z]
            grad_p = [y * z + 2.0 * x * y * y * y * z, x * z + 3.0 * x * x * y * y * z, x * y + x * x * y * y * y]
            # grad eta = -Beta eta (1 - 2 x_i)
            grad_eta = [-b * eta * (1.0 - 2.0 * c) for c in (x, y, z)]
            self._finish(eta, u, p, e, div_e, grad_p, grad_eta)


# ---------------------------------------------------------------------------
# Compilation to a register program evaluated by one kernel (csrc/uwg_fn.cu)
# ---------------------------------------------------------------------------
_OPS = {"const": 0, "input": 1, "add": 2, "sub": 3, "mul": 4, "div": 5, "pow": 6, "max": 7, "min": 8,
        "lt": 9, "le": 10, "gt": 11, "ge": 12, "and": 13, "or": 14, "xor": 15, "neg": 16, "abs": 17,
        "exp": 18, "log": 19, "log2": 20, "log10": 21, "sqrt": 22, "sin": 23, "cos": 24, "tan": 25,
        "asin": 26, "acos": 27, "atan": 28, "sinh": 29, "cosh": 30, "tanh": 31, "asinh": 32, "acosh": 33,
        "atanh": 34, "erf": 35, "erfc": 36, "eqk": 37, "select": 38, "check": 39, "out": 40, "copy": 41,
        "finite": 42}
_BIN_OPS = {torch.add: "add", torch.sub: "sub", torch.mul: "mul", torch.div: "div", torch.pow: "pow",
            torch.maximum: "max", torch.minimum: "min"}
_UN_OPS = {torch.neg: "neg", torch.abs: "abs", torch.exp: "exp", torch.log: "log", torch.log2: "log2",
           torch.log10: "log10", torch.sqrt: "sqrt", torch.sin: "sin", torch.cos: "cos", torch.tan: "tan",
           torch.asin: "asin", torch.acos: "acos", torch.atan: "atan", torch.sinh: "sinh", torch.cosh: "cosh",
           torch.tanh: "tanh", torch.asinh: "asinh", torch.acosh: "acosh", torch.atanh: "atanh",
           torch.erf: "erf", torch.erfc: "erfc"}
_DTYPES = {torch.float64: 0, torch.float32: 1, torch.int32: 2, torch.int8: 3, torch.int16: 4, torch.int64: 5}
# error-check codes of the program and the exceptions they raise on the host
_CHECKS = {0: (RuntimeError, _NO_KEY),
           1: (RuntimeError, _NO_CLAUSE),
           2: (RuntimeError, "Function evaluation produced a non-finite value (SafeMaths).")}


class _Unsupported(Exception):
    pass


class _Program:
    """A function graph lowered to register operations (memoised per node)."""

    MAX_REG = 128

    def __init__(self, ctx):
        self.ctx = ctx
        self.ops = []
        self.inputs = []          # (tensor, by_particle)
        self.nreg = 0
        self.memo = {}

    def reg(self):
        if self.nreg >= self.MAX_REG:
            raise _Unsupported("too many registers")
        self.nreg += 1
        return self.nreg - 1

    def emit(self, op, dst=-1, a=-1, b=-1, imm=0.0):
        self.ops.append((_OPS[op], dst, a, b, float(imm)))
        return dst

    def input(self, t, by_particle):
        if t.dim() == 1:
            t = t[:, None]
        t = t.contiguous()
        if t.dtype not in _DTYPES:
            t = t.double()
        self.inputs.append((t, by_particle))
        slot = len(self.inputs) - 1
        return [self.emit("input", self.reg(), slot, k) for k in range(t.shape[1])]

    @staticmethod
    def _broadcast(a, b):
        if len(a) == len(b):
            return a, b
        if len(a) == 1:
            return a * len(b), b
        if len(b) == 1:
            return a, b * len(a)
        raise _Unsupported("component counts %d and %d" % (len(a), len(b)))

    def node(self, f):
        key = id(f)
        if key not in self.memo:
            self.memo[key] = self._node(f)
        return self.memo[key]

    def _node(self, f):
        if isinstance(f, constant):
            vals = np.atleast_1d(np.asarray(f.value, dtype=np.float64)).ravel()
            return [self.emit("const", self.reg(), imm=v) for v in vals]
        if isinstance(f, _Vector):
            return [r for p in f.parts for r in self.node(p)]
        if isinstance(f, _Bin):
            name = getattr(f, "name", None) or _BIN_OPS.get(f.op)
            if name is None:
                raise _Unsupported("binary operation")
            a, b = self.node(f.a), self.node(f.b)
            if name == "dot":
                a, b = self._broadcast(a, b)
                acc = self.emit("mul", self.reg(), a[0], b[0])
                for x, y in zip(a[1:], b[1:]):
                    t = self.emit("mul", self.reg(), x, y)
                    acc = self.emit("add", self.reg(), acc, t)
                return [acc]
            a, b = self._broadcast(a, b)
            return [self.emit(name, self.reg(), x, y) for x, y in zip(a, b)]
        if isinstance(f, _Bool):
            if f.name is None:
                raise _Unsupported("comparison")
            a, b = self._broadcast(self.node(f.a), self.node(f.b))
            return [self.emit(f.name, self.reg(), x, y) for x, y in zip(a, b)]
        if isinstance(f, _Un):
            name = _UN_OPS.get(f.op)
            if name is None:
                raise _Unsupported("unary operation")
            return [self.emit(name, self.reg(), x) for x in self.node(f.a)]
        if isinstance(f, _Index):
            return [self.node(f.a)[f.i]]
        if isinstance(f, input):
            return self.input(self.ctx.coords, False)
        if isinstance(f, _SwarmVar):
            return self.input(f.var._device_data(), True)
        if isinstance(f, _MeshVar):
            return self.input(f._eval(self.ctx), False)      # sampled by the interpolation kernel
        if isinstance(f, _MeshGrad):
            return self.input(f._eval(self.ctx), False)
        if isinstance(f, _ParticleFound):
            return self.input(f._eval(self.ctx), False)
        if isinstance(f, _Map):
            key = self.node(f.key)[0]
            entries = [(k, self.node(v)) for k, v in f.mapping.items()]
            k = max([len(v) for _, v in entries] + ([len(self.node(f.default))] if f.default is not None else []))
            if f.default is not None:
                out = [self.emit("copy", self.reg(), r) for r in self._broadcast(self.node(f.default), [0] * k)[0]]
                hit = None
            else:
                out = [self.emit("const", self.reg(), imm=float("nan")) for _ in range(k)]
                hit = self.emit("const", self.reg(), imm=0.0)
            for kv, v in entries:
                eq = self.emit("eqk", self.reg(), key, imm=kv)
                v = self._broadcast(v, [0] * k)[0]
                out = [self.emit("select", self.reg(), x, o, imm=eq) for x, o in zip(v, out)]
                if hit is not None:
                    hit = self.emit("or", self.reg(), hit, eq)
            if hit is not None:
                self.emit("check", -1, hit, 0)
            return out
        if isinstance(f, _Conditional):
            clauses = [(self.node(c)[0], self.node(v)) for c, v in f.clauses]
            k = max(len(v) for _, v in clauses)
            out = [self.emit("const", self.reg(), imm=float("nan")) for _ in range(k)]
            done = self.emit("const", self.reg(), imm=0.0)
            for c, v in reversed(clauses):
                v = self._broadcast(v, [0] * k)[0]
                out = [self.emit("select", self.reg(), x, o, imm=c) for x, o in zip(v, out)]
                done = self.emit("or", self.reg(), done, c)
            self.emit("check", -1, done, 1)
            return out
        if isinstance(f, _SafeMaths):
            regs = self.node(f.a)
            for r in regs:
                self.emit("finite", -1, r, 2)
            return regs
        raise _Unsupported(type(f).__name__)


def _eval_kernel(f, ctx, ncomp=None, out=None):
    """Evaluate f at the points of ctx with one kernel launch; returns None when
    the graph holds a node kind the program does not cover.  With `out` (a
    per-particle [n_particles, k] float64 tensor) the values are scattered into
    particle order by the kernel itself."""
    lib_ctx = getattr(ctx, "lib_ctx", None)
    if lib_ctx is None or getattr(ctx, "pid32", None) is None:
        return None
    prog = _Program(ctx)
    try:
        regs = prog.node(f)
    except _Unsupported:
        return None
    k = len(regs)
    if ncomp is not None and k not in (1, ncomp):
        raise ValueError("function returns %d components, %d expected" % (k, ncomp))
    nout = ncomp or k
    regs = regs * nout if k == 1 else regs
    for c, r in enumerate(regs):
        prog.emit("out", c, r)
    res = torch.empty((ctx.n, nout), dtype=torch.float64, device=ctx.device) if out is None else out
    flags = lib_ctx.fn_eval(prog.ops, prog.inputs, ctx.n, ctx.pid32, nout, res, out is not None)
    for code, (exc, msg) in _CHECKS.items():
        if flags & (1 << code):
            raise exc(msg)
    return res


def _input_context(inputData):
    """EvalContext for Function.evaluate: coordinates, a mesh's nodes or a swarm's particles."""
    dev = torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")
    if hasattr(inputData, "particleCoordinates") and hasattr(inputData, "_x"):
        x = inputData._x if inputData._x is not None else torch.zeros((0, inputData.dim), dtype=torch.float64)
        dev = x.device
        ctx = EvalContext(torch.arange(x.shape[0], device=dev), lambda: x, dev)
        ctx.swarm = inputData
        return ctx
    if hasattr(inputData, "_axes") and hasattr(inputData, "elementRes"):
        pts = np.asarray(inputData.data, dtype=np.float64)
    elif hasattr(inputData, "object") and hasattr(getattr(inputData, "object"), "_axes"):
        # a mesh's vertex set: its vertices (FeMesh_IndexSet as a FunctionInput)
        pts = np.asarray(inputData.object.data, dtype=np.float64)[inputData.data.astype(np.int64)]
    else:
        if inputData is None:
            pts = np.zeros((1, 1))
        elif isinstance(inputData, numbers.Number):
            pts = np.array([[float(inputData)]])
        else:
            pts = np.asarray(inputData, dtype=np.float64)
            if pts.ndim == 1:
                pts = pts[None, :]
        t = torch.from_numpy(np.ascontiguousarray(pts)).to(dev)
        ctx = EvalContext(torch.full((t.shape[0],), -1, dtype=torch.int64, device=dev), lambda: t, dev)
        ctx.check_domain = True      # user coordinates: mesh variables refuse points outside their mesh
        return ctx
    t = torch.from_numpy(np.ascontiguousarray(pts)).to(dev)
    return EvalContext(torch.full((t.shape[0],), -1, dtype=torch.int64, device=dev), lambda: t, dev)


from . import _analytic_series as _series  # noqa: E402  (it builds on the classes above)

for _name in ("SolA", "SolB", "SolC", "SolCx", "SolDA", "SolH", "SolKx", "SolKz", "SolM", "SolNL"):
    setattr(analytic, _name, getattr(_series, _name))
del _name
