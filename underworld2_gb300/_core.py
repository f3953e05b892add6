"""Device-side state and thin wrappers over the libuwg C ABI.

``Context`` owns one libuwg context (mesh geometry, assembled operators,
solver workspaces) and ``SwarmState`` the particle arrays of one swarm.
PyTorch is used only to hold device memory and to name the CUDA stream.
"""
import ctypes

import numpy as np
import torch

from . import _native

_MASK = 123459876


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def host_array(shape, dtype):
    """Zeroed numpy array in page-locked host memory when a GPU is visible (copies
    to and from the device then run at DMA speed, without a staging copy), plain
    numpy memory otherwise.  The array keeps its backing tensor alive."""
    if torch.cuda.is_available():
        t = torch.zeros(tuple(shape), dtype=torch.from_numpy(np.zeros(0, dtype=dtype)).dtype, pin_memory=True)
        return t.numpy()
    return np.zeros(shape, dtype=dtype)


def _require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("underworld2_gb300 needs a CUDA GPU (sm_103a); none is visible")


class Context:
    """One regular Cartesian Q1/dQ0 mesh on the current CUDA device."""

    def __init__(self, dim, res, minc, maxc, order=1, porder=0, device=None):
        _require_cuda()
        self.L = _native.load()
        self.device = torch.device(device or "cuda")
        d = _native.MeshDesc()
        d.dim, d.order, d.porder = dim, order, porder
        for i in range(3):
            d.res[i] = int(res[i]) if i < dim else 1
            d.minc[i] = float(minc[i]) if i < dim else 0.0
            d.maxc[i] = float(maxc[i]) if i < dim else 1.0
        self.desc = d
        self.dim, self.order, self.porder = dim, order, porder
        self.res = tuple(int(r) for r in res[:dim])
        self.minc = tuple(float(v) for v in minc[:dim])
        self.maxc = tuple(float(v) for v in maxc[:dim])
        with torch.cuda.device(self.device):
            torch.cuda.current_stream().synchronize()
            h = _native._CTX()
            rc = self.L.uwg_ctx_create(ctypes.byref(d), ctypes.byref(h))
            if rc != 0:
                raise _native.UwgError(rc, "uwg_ctx_create failed (dim=%d order=%d porder=%d res=%s)"
                                       % (dim, order, porder, self.res))
            self.h = h
        sizes = np.zeros(8, np.int64)
        self.L.uwg_mesh_sizes(self.h, ctypes.c_void_p(sizes.ctypes.data))
        self.n_el, self.n_nodes, self.n_vdof, self.n_pdof, self.nen, self.npn, self.nlev = (int(v) for v in sizes[:7])
        self.axes = []
        for a in range(dim):
            buf = np.zeros(self.res[a] * order + 1)
            self.L.uwg_mesh_axis(self.h, a, ctypes.c_void_p(buf.ctypes.data))
            self.axes.append(buf)
        # minimum node separation (as the library computes it: closest adjacent pair on an axis)
        self.min_sep = min(float(np.min(np.sqrt(np.diff(a) ** 2))) for a in self.axes)

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.L.uwg_ctx_destroy(self.h)
                self.h = None
        except Exception:
            pass

    # -- helpers -------------------------------------------------------------
    def _stream(self):
        s = torch.cuda.current_stream(self.device).cuda_stream
        self.L.uwg_set_stream(self.h, ctypes.c_void_p(s))

    def _call(self, name, *args):
        self._stream()
        return _native.check(self.h, getattr(self.L, name)(self.h, *args))

    def zeros(self, *shape, dtype=torch.float64):
        return torch.zeros(*shape, dtype=dtype, device=self.device)

    # -- particles -----------------------------------------------------------
    def layout_random(self, ppc, rng_state):
        np_ = self.n_el * ppc
        x = self.zeros(np_, self.dim)
        owner = self.zeros(np_, dtype=torch.int32)
        off = self.zeros(self.n_el + 1, dtype=torch.int32)
        lst = self.zeros(np_, dtype=torch.int32)
        st = ctypes.c_int64(rng_state)
        self._call("uwg_layout_random", int(ppc), ctypes.byref(st), _ptr(x), _ptr(owner), _ptr(off), _ptr(lst))
        return x, owner, off, lst, st.value

    def locate(self, x):
        owner = self.zeros(x.shape[0], dtype=torch.int32)
        self._call("uwg_locate", x.shape[0], _ptr(x), _ptr(owner))
        return owner

    def gauss_nearest(self, xi_q, off, lst, x):
        """Particle index of each Gauss point (element-major), -1 in empty elements."""
        xi_q = xi_q.to(device=self.device, dtype=torch.float64).contiguous()
        x = x.to(torch.float64).contiguous()
        pid = self.zeros(self.n_el * xi_q.shape[0], dtype=torch.int32)
        self._call("uwg_gauss_nearest", xi_q.shape[0], _ptr(xi_q), _ptr(off), _ptr(lst), _ptr(x), _ptr(pid))
        return pid

    def update_owners(self, x, owner, off, lst):
        """Owner update; x may be stored in FP64 or FP32."""
        lost = ctypes.c_int64(0)
        name = "uwg_update_owners_f32" if x.dtype == torch.float32 else "uwg_update_owners"
        self._call(name, x.shape[0], _ptr(x), _ptr(owner), _ptr(off), _ptr(lst), ctypes.byref(lost))
        return lost.value

    def pic_map(self, x, off, lst):
        ip_xi = self.zeros(x.shape[0], self.dim)
        self._call("uwg_pic_map", x.shape[0], _ptr(x), _ptr(off), _ptr(lst), _ptr(ip_xi))
        return ip_xi

    def dvc_weights(self, off, ip_xi, res=15):
        ip_w = self.zeros(ip_xi.shape[0])
        self._call("uwg_dvc_weights", int(res), _ptr(off), _ptr(ip_xi), _ptr(ip_w))
        return ip_w

    # -- particle deletion and creation ---------------------------------------
    def pop_plan_escaped(self, owner, off, lst):
        n = ctypes.c_int64(0)
        self._call("uwg_pop_plan_escaped", owner.shape[0], _ptr(owner), _ptr(off), _ptr(lst), ctypes.byref(n))
        return n.value

    def pop_plan_pcdvc(self, owner, off, lst, ip_w, split_threshold, delete_threshold, max_splits, max_deletions):
        n, ns, nd = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int64(0)
        self._call("uwg_pop_plan_pcdvc", owner.shape[0], _ptr(owner), _ptr(off), _ptr(lst), _ptr(ip_w),
                   float(split_threshold), float(delete_threshold), int(max_splits), int(max_deletions),
                   ctypes.byref(n), ctypes.byref(ns), ctypes.byref(nd))
        return n.value, ns.value, nd.value

    def pop_apply(self, ip_xi, x_old, np_new):
        """Apply the pending plan: new (x, owner, cell_offsets, cell_list) and the
        old index whose data each new particle carries (host int64)."""
        x = self.zeros(np_new, self.dim)
        owner = self.zeros(np_new, dtype=torch.int32)
        off = self.zeros(self.n_el + 1, dtype=torch.int32)
        lst = self.zeros(np_new, dtype=torch.int32)
        src = np.zeros(np_new, np.int64)
        self._call("uwg_pop_apply", _ptr(ip_xi), _ptr(x_old), _ptr(x), _ptr(owner), _ptr(off), _ptr(lst),
                   ctypes.c_void_p(src.ctypes.data))
        return x, owner, off, lst, src

    # -- assembly and solve ----------------------------------------------------
    def set_bcs(self, mask, values=None):
        mask = mask.to(self.device, torch.uint8).contiguous()
        values = None if values is None else values.to(self.device, torch.float64).contiguous()
        self._call("uwg_set_bcs", _ptr(mask), _ptr(values))

    def assemble(self, off, lst, ip_xi, ip_w, eta, body=None, one_on_lambda=None):
        self._call("uwg_assemble", lst.shape[0], _ptr(off), _ptr(lst), _ptr(ip_xi), _ptr(ip_w), _ptr(eta),
                   _ptr(body), _ptr(one_on_lambda))

    def add_force(self, df):
        """f += df at free dofs (traction surface term; after assemble)."""
        self._call("uwg_add_force", _ptr(df.contiguous()))

    def fn_eval(self, ops, inputs, n, pid32, nout, out, by_particle):
        """Run a compiled function program (function.py) at n points; returns the check flags."""
        from . import function as _fn
        arr = (_native.FnOp * max(len(ops), 1))(*[_native.FnOp(*o) for o in ops])
        ins = (_native.FnInput * max(len(inputs), 1))(
            *[_native.FnInput(t.data_ptr(), _fn._DTYPES[t.dtype], t.shape[1], int(bp), 0) for t, bp in inputs])
        flags = ctypes.c_int32(0)
        self._call("uwg_fn_eval", len(ops), ctypes.cast(arr, ctypes.c_void_p), len(inputs),
                   ctypes.cast(ins, ctypes.c_void_p), int(n), _ptr(pid32), int(nout), int(bool(by_particle)),
                   _ptr(out), ctypes.byref(flags))
        return flags.value

    def add_source(self, off, lst, ip_xi, ip_w, src):
        """h += the continuity source term from per-particle values (after assemble)."""
        self._call("uwg_add_source", _ptr(off), _ptr(lst), _ptr(ip_xi), _ptr(ip_w), _ptr(src.contiguous()))

    def element_matrices(self, el):
        nd = self.dim * self.nen
        Ke = np.zeros((nd, nd))
        fe = np.zeros(nd)
        Ge = np.zeros((nd, self.npn))
        Se = np.zeros((self.npn, self.npn))
        p = lambda a: ctypes.c_void_p(a.ctypes.data)
        self._call("uwg_element_matrices", int(el), p(Ke), p(fe), p(Ge), p(Se))
        return Ke, Ge, Se

    def solve(self, u, p, **opts):
        o = _native.SolveOpts()
        self.L.uwg_solve_opts_default(ctypes.byref(o))
        for k, v in opts.items():
            if not hasattr(o, k):
                raise ValueError("unknown solver option %r" % k)
            setattr(o, k, v)
        st = _native.SolveStats()
        self._call("uwg_stokes_solve", ctypes.byref(o), _ptr(u), _ptr(p), ctypes.byref(st))
        return st.as_dict()

    def residuals(self, u, p):
        out = np.zeros(2)
        self._call("uwg_stokes_residuals", _ptr(u), _ptr(p), ctypes.c_void_p(out.ctypes.data))
        return out

    def apply_K(self, x, level=0):
        y = torch.empty_like(x)
        self._call("uwg_apply_K64" if x.dtype == torch.float64 else "uwg_apply_K32", int(level), _ptr(x), _ptr(y))
        return y

    def apply_K_refine(self, x):
        """The refinement-residual operator (FP64 input and output)."""
        y = torch.empty_like(x)
        self._call("uwg_apply_K_refine", _ptr(x), _ptr(y))
        return y

    def apply_G(self, p):
        y = self.zeros(self.n_vdof)
        self._call("uwg_apply_G", _ptr(p), _ptr(y))
        return y

    def apply_Gt(self, u):
        q = self.zeros(self.n_pdof)
        self._call("uwg_apply_Gt", _ptr(u), _ptr(q))
        return q

    # -- advection -------------------------------------------------------------
    def rk2(self, x, vel, dt):
        """Midpoint RK2 in FP64; x may be stored in FP64 or FP32 (rounded once per step)."""
        fb, failed = ctypes.c_int64(0), ctypes.c_int64(0)
        name = "uwg_rk2_advect_f32" if x.dtype == torch.float32 else "uwg_rk2_advect"
        self._call(name, x.shape[0], float(dt), _ptr(vel), _ptr(x), ctypes.byref(fb), ctypes.byref(failed))
        return fb.value, failed.value

    def interpolate(self, pts, vel):
        out = torch.empty_like(pts)
        self._call("uwg_interpolate", pts.shape[0], _ptr(pts), _ptr(vel), _ptr(out))
        return out

    def interpolate_field(self, pts, field, ncomp, grad=False):
        """Values [n, ncomp] (and gradients [n, ncomp, dim]) of a nodal field at points."""
        out = torch.empty((pts.shape[0], ncomp), dtype=torch.float64, device=self.device)
        g = torch.empty((pts.shape[0], ncomp, self.dim), dtype=torch.float64, device=self.device) if grad else None
        self._call("uwg_interpolate_field", pts.shape[0], _ptr(pts), _ptr(field), int(ncomp), _ptr(out), _ptr(g))
        return out, g

    def max_dt(self, vel):
        dt = ctypes.c_double(0.0)
        self._call("uwg_max_dt", _ptr(vel), ctypes.byref(dt))
        return dt.value

    # -- SUPG advection-diffusion --------------------------------------------
    def gauss_coords(self, n=3):
        """Global coordinates of the n^dim Gauss points (n = 3 or 5) of every
        element, [n_el * n^dim, dim] on the device (x-fastest points, element
        order, ascending abscissae)."""
        g1 = gauss_abscissae(n)
        pts = np.stack(np.meshgrid(*([g1] * self.dim), indexing="ij"), axis=-1).reshape(-1, self.dim)
        pts = pts[:, ::-1] if self.dim > 1 else pts                    # x fastest
        ex = np.indices(self.res[::-1]).reshape(self.dim, -1)[::-1].T   # element index grid, x fastest
        out = np.zeros((self.n_el, len(pts), self.dim))
        for d in range(self.dim):
            a = self.axes[d]
            lo, hi = a[ex[:, d]], a[ex[:, d] + 1]
            out[:, :, d] = lo[:, None] + 0.5 * (pts[None, :, d] + 1.0) * (hi - lo)[:, None]
        return torch.from_numpy(out.reshape(-1, self.dim)).to(self.device)

    def advdiff_step(self, dt, vel, kappa_q, phi, phidot, bc, bcval, bcdot=None, source_q=None, iterations=2,
                     gamma=0.5, flux=None):
        bc = bc.to(self.device, torch.uint8).contiguous()
        self._call("uwg_advdiff_step", float(dt), _ptr(vel), _ptr(kappa_q), _ptr(source_q), _ptr(bc), _ptr(bcval),
                   _ptr(bcdot), _ptr(phi), _ptr(phidot), int(iterations), float(gamma), _ptr(flux))

    def advdiff_max_dt(self, vel, kappa_q, courant=0.5):
        dt = ctypes.c_double(0.0)
        self._call("uwg_advdiff_max_dt", _ptr(vel), _ptr(kappa_q), float(courant), ctypes.byref(dt))
        return dt.value

    # -- SLCN advection-diffusion --------------------------------------------
    def slcn_phistar(self, dt, vel, phi):
        out = torch.empty_like(phi)
        self._call("uwg_slcn_phistar", float(dt), _ptr(vel), _ptr(phi), _ptr(out))
        return out

    def slcn_solve(self, dt, kappa_q, bc, phistar, phi, source_q=None, rtol=1e-10, max_its=5000, flux=None):
        bc = bc.to(self.device, torch.uint8).contiguous()
        its, res = ctypes.c_int(0), ctypes.c_double(0.0)
        self._call("uwg_slcn_solve", float(dt), _ptr(kappa_q), _ptr(source_q), _ptr(bc), _ptr(phistar), _ptr(phi),
                   float(rtol), int(max_its), ctypes.byref(its), ctypes.byref(res), _ptr(flux))
        return its.value, res.value


def gauss_abscissae(n):
    """Ascending Gauss-Legendre abscissae on [-1, 1] for n = 3 or 5, in the
    closed forms the library uses."""
    if n == 3:
        x = np.sqrt(0.6)
        return np.array([-x, 0.0, x])
    if n == 5:
        a = np.sqrt(5.0 - 2.0 * np.sqrt(10.0 / 7.0)) / 3.0
        b = np.sqrt(5.0 + 2.0 * np.sqrt(10.0 / 7.0)) / 3.0
        return np.array([-b, -a, 0.0, a, b])
    raise ValueError("Gauss rules of 3 or 5 points per axis are provided")


def rng_seed(seed):
    """Park-Miller state after Swarm_Random_Seed (L/StgDomain/Swarm/src/Random.c:37-40)."""
    return int(seed) ^ _MASK
