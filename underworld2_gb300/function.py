"""The subset of ``underworld.function`` that the PIC Stokes path needs.

Functions are small expression trees evaluated once per integration point
into arrays (viscosity, body force, compressibility), on the device with
torch tensor arithmetic, mirroring the reference's per-point evaluation
(``SwarmVariableFn::getFunction`` maps an integration point to its material
particle, L/Underworld/Function/src/SwarmVariableFn.cpp:30-110; coordinate
inputs are the integration point's global position).

Supported: constants and tuples, ``input()``/``coord()``, swarm and mesh
variables, arithmetic (+ - * / **, unary -), comparisons and logical
and/or, ``math.exp/log/sqrt/sin/cos/abs/pow/dot``, ``branching.map`` and
``branching.conditional``.
"""
import numbers

import torch


class EvalContext:
    """Where to evaluate: integration points with their particle ids and
    global coordinates (coords computed on demand)."""

    def __init__(self, particle_ids, coords_fn, device):
        self.pid = particle_ids
        self._coords_fn = coords_fn
        self._coords = None
        self.device = device

    @property
    def coords(self):
        if self._coords is None:
            self._coords = self._coords_fn()
        return self._coords

    @property
    def n(self):
        return self.pid.shape[0]


class Function:
    """Base class: ``_eval(ctx)`` returns a float64 tensor of shape (n, k)."""

    @staticmethod
    def convert(obj):
        if obj is None or isinstance(obj, Function):
            return obj
        if isinstance(obj, numbers.Number):
            return constant(obj)
        if isinstance(obj, (tuple, list)):
            parts = [Function.convert(o) for o in obj]
            if all(isinstance(p, constant) for p in parts):
                return constant([p.value for p in parts])
            return _Vector(parts)
        if hasattr(obj, "_as_function"):
            return obj._as_function()
        raise TypeError("cannot convert %r to a Function" % (obj,))

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
    def __lt__(self, o): return _Bin(lambda a, b: (a < b).double(), self, Function.convert(o))
    def __le__(self, o): return _Bin(lambda a, b: (a <= b).double(), self, Function.convert(o))
    def __gt__(self, o): return _Bin(lambda a, b: (a > b).double(), self, Function.convert(o))
    def __ge__(self, o): return _Bin(lambda a, b: (a >= b).double(), self, Function.convert(o))
    def __and__(self, o): return _Bin(lambda a, b: ((a != 0) & (b != 0)).double(), self, Function.convert(o))
    def __or__(self, o): return _Bin(lambda a, b: ((a != 0) | (b != 0)).double(), self, Function.convert(o))

    def __getitem__(self, i):
        return _Index(self, i)


class constant(Function):
    def __init__(self, value):
        self.value = value

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

    def _children(self):
        return [self.a, self.b]

    def _eval(self, ctx):
        return self.op(self.a.evaluate_at(ctx), self.b.evaluate_at(ctx))


class _Un(Function):
    def __init__(self, op, a):
        self.op, self.a = op, a

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

    def _eval(self, ctx):
        d = self.var._device_data()
        if d.dim() == 1:
            d = d[:, None]
        return d[ctx.pid.long()].double()

    def depends_on(self, kinds):
        return "swarm" in kinds


class _MeshVar(Function):
    def __init__(self, var):
        self.var = var

    def _eval(self, ctx):
        return self.var._interpolate(ctx.coords)

    def depends_on(self, kinds):
        return "coord" in kinds or "mesh" in kinds


class math:
    @staticmethod
    def exp(f): return _Un(torch.exp, Function.convert(f))

    @staticmethod
    def log(f): return _Un(torch.log, Function.convert(f))

    @staticmethod
    def sqrt(f): return _Un(torch.sqrt, Function.convert(f))

    @staticmethod
    def sin(f): return _Un(torch.sin, Function.convert(f))

    @staticmethod
    def cos(f): return _Un(torch.cos, Function.convert(f))

    @staticmethod
    def abs(f): return _Un(torch.abs, Function.convert(f))

    @staticmethod
    def pow(a, b): return _Bin(torch.pow, Function.convert(a), Function.convert(b))

    @staticmethod
    def dot(a, b):
        return _Bin(lambda x, y: (x * y).sum(dim=1, keepdim=True), Function.convert(a), Function.convert(b))


class _Map(Function):
    def __init__(self, fn_key, mapping, fn_default=None):
        self.key = Function.convert(fn_key)
        self.mapping = {int(k): Function.convert(v) for k, v in mapping.items()}
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
            raise ValueError("branching.map: a key has no mapping and no default is given")
        return out


class _Conditional(Function):
    def __init__(self, clauses):
        self.clauses = [(Function.convert(c), Function.convert(v)) for c, v in clauses]

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
            raise RuntimeError("branching.conditional: no clause evaluated true for some points")
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
