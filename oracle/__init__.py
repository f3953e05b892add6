"""CPU oracle for the particle-in-cell Stokes path -- TEST INFRASTRUCTURE.

The C restatement in ``uwo.c`` follows the reference's algorithms line by
line (citations inside).  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` may import this package; the library in
``underworld2_gb300`` never does.

``build()`` compiles ``uwo.c`` with ``gcc -O2 -ffp-contract=off -fopenmp``
into ``oracle/_build/libuwo.so``; :func:`lib` loads it through ctypes and
:class:`Mesh` wraps the plain-array entry points with numpy.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "libuwo.so")
_lib = None


def build(force=False):
    """Compile the oracle (seconds).  Rebuilds when the source is newer."""
    srcs = [os.path.join(_HERE, f) for f in ("uwo.c", "uwo_solve.c")]
    os.makedirs(_BUILD, exist_ok=True)
    if not force and os.path.exists(_SO) and all(os.path.getmtime(_SO) >= os.path.getmtime(s) for s in srcs):
        return _SO
    tmp = _SO + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=c11",
           "-o", tmp] + srcs + ["-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, _SO)
    return _SO


class _MeshC(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int), ("order", ctypes.c_int), ("res", ctypes.c_int * 3),
                ("minc", ctypes.c_double * 3), ("maxc", ctypes.c_double * 3)]


_P = ctypes.c_void_p
_I64 = ctypes.c_int64


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_SO)
        M = ctypes.POINTER(_MeshC)
        sig = {
            "uwo_axis_coords": (None, [M, ctypes.c_int, _P]),
            "uwo_element_nodes": (None, [M, _I64, _P]),
            "uwo_rng_seed": (_I64, [_I64]),
            "uwo_layout_random": (_I64, [M, _P, _P, _P, ctypes.c_int, _I64, _P]),
            "uwo_search_element": (ctypes.c_int, [M, _P, _P]),
            "uwo_cell_of": (_I64, [M, _P]),
            "uwo_global_to_local": (ctypes.c_int, [M, _P, _P, _P, _I64, _P, _P]),
            "uwo_update_owners": (_I64, [M, _I64, _P, _P, _P, _P, ctypes.c_int]),
            "uwo_dvc_element": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, _P]),
            "uwo_pic_map": (None, [M, _P, _P, _P, _P, _P, _P, ctypes.c_int, _I64, _I64, ctypes.c_int, _P, _P]),
            "uwo_element_K": (None, [M, _P, _P, _P, _I64, ctypes.c_int, _P, _P, _P, _P]),
            "uwo_element_G": (None, [M, _P, _P, _P, ctypes.c_int, _I64, ctypes.c_int, _P, _P, _P]),
            "uwo_element_f": (None, [M, _P, _P, _P, _I64, ctypes.c_int, _P, _P, _P, _P]),
            "uwo_element_M": (None, [M, _P, _P, _P, ctypes.c_int, _I64, ctypes.c_int, _P, _P, _P, _P]),
            "uwo_element_h": (None, [M, _P, _P, _P, ctypes.c_int, _I64, ctypes.c_int, _P, _P, _P, _P]),
            "uwo_element_S": (None, [ctypes.c_int, ctypes.c_int, _P, _P, _P]),
            "uwo_shape": (None, [ctypes.c_int, ctypes.c_int, _P, _P, _P]),
            "uwo_pressure_shape": (None, [ctypes.c_int, ctypes.c_int, _P, _P]),
            "uwo_interpolate": (ctypes.c_int, [M, _P, _P, _P, _P, _P, _P]),
            "uwo_rk2": (None, [M, _P, _P, _P, _P, ctypes.c_double, _I64, _I64, _P, _P]),
            "uwo_slcn_phistar": (ctypes.c_int, [M, _P, _P, _P, _P, _P, ctypes.c_double, ctypes.c_double, _P]),
            "uwo_local_to_global": (None, [M, _P, _P, _P, _I64, _P, _P]),
            "uwo_sys_create": (_P, [ctypes.c_int, _P, _P, _P, _P]),
            "uwo_sys_destroy": (None, [_P]),
            "uwo_sys_set_bc": (None, [_P, _P, _P]),
            "uwo_sys_assemble_points": (None, [_P, _P, _P, _P, _P, _P, _P]),
            "uwo_sys_finish": (None, [_P]),
            "uwo_sys_set_schur_pc": (None, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_double]),
            "uwo_sys_time_iterations": (None, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P]),
            "uwo_sys_applyK": (None, [_P, ctypes.c_int, _P, _P]),
            "uwo_sys_solve": (ctypes.c_int, [_P, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, _P, _P, _P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def gauss_1d(n):
    """Gauss-Legendre abscissae and weights on [-1, 1]."""
    x, w = np.polynomial.legendre.leggauss(n)
    return x, w


class Mesh:
    """Regular Cartesian mesh as the oracle sees it (Q1 or Q2 velocity)."""

    def __init__(self, dim, order, res, minc, maxc, porder=0):
        self.dim, self.order, self.porder = dim, order, porder
        self.res = tuple(int(r) for r in res[:dim])
        self.minc = tuple(float(v) for v in minc[:dim])
        self.maxc = tuple(float(v) for v in maxc[:dim])
        c = _MeshC()
        c.dim, c.order = dim, order
        for d in range(3):
            c.res[d] = self.res[d] if d < dim else 1
            c.minc[d] = self.minc[d] if d < dim else 0.0
            c.maxc[d] = self.maxc[d] if d < dim else 1.0
        self._c = c
        self.L = lib()
        self.axes = []
        for d in range(3):
            n = (c.res[d] * order + 1) if d < dim else 1
            a = np.zeros(n)
            if d < dim:
                self.L.uwo_axis_coords(ctypes.byref(c), d, _p(a))
            self.axes.append(a)
        self.n_el = int(np.prod(self.res))
        self.nen = (order + 1) ** dim
        self.npn = 1 if porder == 0 else (3 if dim == 2 else 4)
        self.n_nodes = int(np.prod([len(a) for a in self.axes[:dim]]))

    def _ax(self):
        return _p(self.axes[0]), _p(self.axes[1]), _p(self.axes[2])

    def element_nodes(self, el):
        out = np.zeros(27, np.int64)
        self.L.uwo_element_nodes(ctypes.byref(self._c), el, _p(out))
        return out[: self.nen]

    def connectivity(self):
        return np.stack([self.element_nodes(e) for e in range(self.n_el)])

    def node_coords(self):
        g = np.meshgrid(*self.axes[: self.dim], indexing="ij")
        return np.stack([x.transpose().ravel() for x in g], axis=1) if self.dim == 2 else \
            np.stack([np.transpose(x, (2, 1, 0)).ravel() for x in g], axis=1)

    # -- particles -------------------------------------------------------
    def layout_random(self, ppc, seed=13, state=None):
        st = self.L.uwo_rng_seed(seed) if state is None else state
        coords = np.zeros((self.n_el * ppc, self.dim))
        st = self.L.uwo_layout_random(ctypes.byref(self._c), *self._ax(), ppc, st, _p(coords))
        return coords, st

    def cell_of(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        return np.array([self.L.uwo_cell_of(ctypes.byref(self._c), _p(x[i])) for i in range(len(x))],
                        dtype=np.int64)

    def global_to_local(self, el, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        xi = np.zeros(3)
        its = self.L.uwo_global_to_local(ctypes.byref(self._c), *self._ax(), int(el), _p(x), _p(xi))
        return xi[: self.dim], its

    def initial_tables(self, ppc, cap):
        nel = self.n_el
        tbl = np.full((nel, cap), -1, np.int32)
        tbl[:, :ppc] = np.arange(nel * ppc, dtype=np.int32).reshape(nel, ppc)
        cnt = np.full(nel, ppc, np.int32)
        owner = np.repeat(np.arange(nel, dtype=np.int32), ppc)
        return tbl, cnt, owner

    def update_owners(self, coords, owner, tbl, cnt):
        coords = np.ascontiguousarray(coords)
        cap = tbl.shape[1]
        lost = self.L.uwo_update_owners(ctypes.byref(self._c), len(coords), _p(coords), _p(owner),
                                        _p(tbl), _p(cnt), cap)
        if lost < 0:
            raise RuntimeError("cell table overflow")
        return lost

    def pic_map(self, coords, tbl, cnt, dvc_res=15):
        n = len(coords)
        ip_xi = np.zeros((n, self.dim))
        ip_w = np.zeros(n)
        self.L.uwo_pic_map(ctypes.byref(self._c), *self._ax(), _p(np.ascontiguousarray(coords)),
                           _p(tbl), _p(cnt), tbl.shape[1], 0, self.n_el, dvc_res, _p(ip_xi), _p(ip_w))
        return ip_xi, ip_w

    def gauss_nearest(self, x, tbl, cnt, xi_q):
        """Particle of every Gauss point, as GeneralSwarm_IntegrationPointMap finds it
        (L/PICellerator/MaterialPoints/src/GeneralSwarm.cpp:319-431): the point's
        global position (FeMesh_CoordLocalToGlobal), then the first particle of the
        element's cell table at the least squared distance; -1 in empty elements.
        Returns [n_el, nq]."""
        xi_q = np.asarray(xi_q, dtype=np.float64)
        key = xi_q.tobytes()
        cache = self.__dict__.setdefault("_gauss_global", {})
        if key not in cache:
            cache[key] = np.array([[self.local_to_global(e, q) for q in xi_q] for e in range(self.n_el)])
        G = cache[key]
        out = np.full((self.n_el, len(xi_q)), -1, dtype=np.int64)
        for e in range(self.n_el):
            if cnt[e] == 0:
                continue
            ps = tbl[e, : cnt[e]]
            g = G[e]
            d2 = np.zeros((len(xi_q), len(ps)))
            for d in range(self.dim):
                dd = g[:, d][:, None] - x[ps, d][None, :]
                d2 = d2 + dd * dd
            out[e] = ps[np.argmin(d2, axis=1)]
        return out

    # -- element terms ---------------------------------------------------
    def element_K(self, el, xi, w, eta):
        nd = self.dim * self.nen
        Ke = np.zeros((nd, nd))
        xi = np.ascontiguousarray(xi, np.float64)
        self.L.uwo_element_K(ctypes.byref(self._c), *self._ax(), int(el), len(w), _p(xi),
                             _p(np.ascontiguousarray(w, np.float64)),
                             _p(np.ascontiguousarray(eta, np.float64)), _p(Ke))
        return Ke

    def element_G(self, el, xi, w):
        Ge = np.zeros((self.dim * self.nen, self.npn))
        self.L.uwo_element_G(ctypes.byref(self._c), *self._ax(), self.porder, int(el), len(w),
                             _p(np.ascontiguousarray(xi, np.float64)),
                             _p(np.ascontiguousarray(w, np.float64)), _p(Ge))
        return Ge

    def element_f(self, el, xi, w, fq):
        fe = np.zeros(self.dim * self.nen)
        self.L.uwo_element_f(ctypes.byref(self._c), *self._ax(), int(el), len(w),
                             _p(np.ascontiguousarray(xi, np.float64)),
                             _p(np.ascontiguousarray(w, np.float64)),
                             _p(np.ascontiguousarray(fq, np.float64)), _p(fe))
        return fe

    def element_M(self, el, xi, w, Fq):
        Me = np.zeros((self.npn, self.npn))
        self.L.uwo_element_M(ctypes.byref(self._c), *self._ax(), self.porder, int(el), len(w),
                             _p(np.ascontiguousarray(xi, np.float64)),
                             _p(np.ascontiguousarray(w, np.float64)),
                             _p(np.ascontiguousarray(Fq, np.float64)), _p(Me))
        return Me

    def element_h(self, el, xi, w, Fq):
        he = np.zeros(self.npn)
        self.L.uwo_element_h(ctypes.byref(self._c), *self._ax(), self.porder, int(el), len(w),
                             _p(np.ascontiguousarray(xi, np.float64)),
                             _p(np.ascontiguousarray(w, np.float64)),
                             _p(np.ascontiguousarray(Fq, np.float64)), _p(he))
        return he

    def element_S(self, Ke, Ge):
        Se = np.zeros((self.npn, self.npn))
        self.L.uwo_element_S(Ke.shape[0], self.npn, _p(np.ascontiguousarray(Ke)),
                             _p(np.ascontiguousarray(Ge)), _p(Se))
        return Se

    def gauss_points(self, n=None):
        if n is None:
            n = 3 if self.order == 1 else 5
        x, w = gauss_1d(n)
        if self.dim == 2:
            xi = np.array([[x[i], x[j]] for j in range(n) for i in range(n)])
            wt = np.array([w[i] * w[j] for j in range(n) for i in range(n)])
        else:
            xi = np.array([[x[i], x[j], x[k]] for k in range(n) for j in range(n) for i in range(n)])
            wt = np.array([w[i] * w[j] * w[k] for k in range(n) for j in range(n) for i in range(n)])
        return xi, wt

    # -- advection ---------------------------------------------------------
    def rk2(self, vel, dt, coords):
        coords = np.ascontiguousarray(coords, np.float64)
        counts = np.zeros(2, np.int64)
        self.L.uwo_rk2(ctypes.byref(self._c), *self._ax(), _p(np.ascontiguousarray(vel, np.float64)),
                       float(dt), 0, len(coords), _p(coords), _p(counts))
        return coords, counts

    def local_to_global(self, el, xi):
        x = np.zeros(3)
        self.L.uwo_local_to_global(ctypes.byref(self._c), *self._ax(), int(el),
                                   _p(np.ascontiguousarray(xi, np.float64)), _p(x))
        return x[: self.dim]

    def min_sep(self):
        """Mesh minimum separation: the closest adjacent node pair along an axis."""
        return min(float(np.min(np.sqrt(np.diff(a) ** 2))) for a in self.axes[: self.dim])

    def slcn_phistar(self, vel, phi, dt):
        out = np.zeros(self.n_nodes)
        rc = self.L.uwo_slcn_phistar(ctypes.byref(self._c), *self._ax(), _p(np.ascontiguousarray(vel, np.float64)),
                                     _p(np.ascontiguousarray(phi, np.float64)), float(dt), self.min_sep(), _p(out))
        if rc != 0:
            raise ValueError("semi-Lagrangian stencils need at least 4 nodes per axis")
        return out

    def interpolate(self, vel, x):
        v = np.zeros(3)
        ok = self.L.uwo_interpolate(ctypes.byref(self._c), *self._ax(),
                                    _p(np.ascontiguousarray(vel, np.float64)),
                                    _p(np.ascontiguousarray(x, np.float64)), _p(v))
        return (v[: self.dim] if ok else None)


def dvc_element(dim, res, xi):
    xi = np.ascontiguousarray(xi, np.float64)
    n = len(xi)
    cx = np.zeros((n, dim))
    w = np.zeros(n)
    rounds = lib().uwo_dvc_element(dim, res, n, _p(xi), _p(cx), _p(w))
    return cx, w, rounds


class StokesCPU:
    """CPU assembly + BSSCR solve on a regular Q1/dQ0 mesh (uwo_solve.c)."""

    def __init__(self, mesh):
        self.mesh = mesh
        L = mesh.L
        res = np.array(list(mesh.res) + [1] * (3 - mesh.dim), np.int32)
        self._res = res
        self.h = L.uwo_sys_create(mesh.dim, _p(res), *mesh._ax())
        self.nv = mesh.n_nodes * mesh.dim
        self.np = mesh.n_el

    def __del__(self):
        try:
            self.mesh.L.uwo_sys_destroy(self.h)
        except Exception:
            pass

    def set_bc(self, mask, values=None):
        mask = np.ascontiguousarray(mask, np.uint8)
        values = None if values is None else np.ascontiguousarray(values, np.float64)
        self.mesh.L.uwo_sys_set_bc(self.h, _p(mask), _p(values))

    def set_schur_pc(self, pc, deg=2, rtol=3e-2):
        """0: the assembled Uzawa term (the reference's "uw"); 1: weighted scaled
        BFBt with the GPU library's pressure multigrid.  Takes effect at assemble."""
        self.mesh.L.uwo_sys_set_schur_pc(self.h, int(pc), int(deg), float(rtol))

    def assemble(self, off, lst, ip_xi, ip_w, eta, body):
        a = [np.ascontiguousarray(off, np.int32), np.ascontiguousarray(lst, np.int32),
             np.ascontiguousarray(ip_xi, np.float64), np.ascontiguousarray(ip_w, np.float64),
             np.ascontiguousarray(eta, np.float64), np.ascontiguousarray(body, np.float64)]
        self.mesh.L.uwo_sys_assemble_points(self.h, *[_p(x) for x in a])
        self.mesh.L.uwo_sys_finish(self.h)

    def time_iterations(self, n_vel=2, n_l=2, deg=2):
        """(seconds per velocity MG-CG iteration, seconds per pressure-Laplacian CG iteration)."""
        out = np.zeros(2)
        self.mesh.L.uwo_sys_time_iterations(self.h, int(n_vel), int(n_l), int(deg), _p(out))
        return float(out[0]), float(out[1])

    def applyK(self, x, level=0):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros_like(x)
        self.mesh.L.uwo_sys_applyK(self.h, level, _p(x), _p(y))
        return y

    def solve(self, inner_rtol=1e-10, outer_rtol=1e-9, max_inner=500, max_outer=500, deg=3):
        u = np.zeros(self.nv)
        p = np.zeros(self.np)
        st = np.zeros(8)
        rc = self.mesh.L.uwo_sys_solve(self.h, inner_rtol, outer_rtol, max_inner, max_outer, deg,
                                       _p(u), _p(p), _p(st))
        return u, p, {"rc": rc, "pressure_its": int(st[0]), "velocity_presolve_its": int(st[1]),
                      "velocity_pressuresolve_its": int(st[2]), "velocity_backsolve_its": int(st[3]),
                      "residual": float(st[4]), "schur_pc_its": int(st[5])}
