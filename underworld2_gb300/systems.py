"""``uw.systems`` drop-ins for the PIC Stokes path: Stokes, Solver/StokesSolver,
SwarmAdvector, AdvectionDiffusion (P/systems/_stokes.py, _solver.py, _bsscr.py,
_timeintegration.py, _advectiondiffusion.py).
"""
import time
import warnings

import numpy as np
import torch

from . import conditions as _cond
from . import function as _fn
from . import mesh as _mesh
from . import swarm as _swarm


class Stokes:
    """The incompressible (or compressible) Stokes system K u + G p = f,
    G^T u + C p = h on a Q1/dQ0 or Q2/dPc1 mesh (P/systems/_stokes.py:106-330)."""

    def __init__(self, velocityField, pressureField, fn_viscosity, fn_bodyforce=None, fn_one_on_lambda=None,
                 fn_source=None, voronoi_swarm=None, conditions=[], gauss_swarm=None, _removeBCs=True,
                 _fn_viscosity2=None, _fn_director=None, fn_stresshistory=None, **kwargs):
        if not isinstance(velocityField, _mesh.MeshVariable):
            raise TypeError("Provided 'velocityField' must be of 'MeshVariable' class.")
        if velocityField.nodeDofCount != velocityField.mesh.dim:
            raise ValueError("Provided 'velocityField' must be a vector field of same dimensionality as its mesh.")
        if not isinstance(pressureField, _mesh.MeshVariable):
            raise TypeError("Provided 'pressureField' must be of 'MeshVariable' class.")
        if pressureField.nodeDofCount != 1:
            raise ValueError("Provided 'pressureField' must be a scalar field (ie pressureField.nodeDofCount==1).")
        for name, v in (("_fn_viscosity2", _fn_viscosity2), ("_fn_director", _fn_director),
                        ("fn_stresshistory", fn_stresshistory)):
            if v is not None:
                raise NotImplementedError("%s is not part of the GPU PIC Stokes path" % name)
        if voronoi_swarm is not None and not isinstance(voronoi_swarm, _swarm.Swarm):
            raise TypeError("Provided 'voronoi_swarm' must be of 'Swarm' class.")
        self._velocityField = velocityField
        self._pressureField = pressureField
        self.mesh = velocityField.mesh
        self.fn_viscosity = fn_viscosity
        if fn_bodyforce is None:
            fn_bodyforce = (0.0,) * self.mesh.dim
        self.fn_bodyforce = fn_bodyforce
        self._fn_one_on_lambda = _fn.Function.convert(fn_one_on_lambda) if fn_one_on_lambda is not None else None
        self._fn_source = None
        self._has_source_term = fn_source is not None
        if fn_source is not None:
            self._fn_source = _fn.Function.convert(fn_source)
            if not isinstance(self._fn_source, _fn.Function):
                raise ValueError("Provided 'fn_source' must be of, or convertible to, the 'Function' class.")
        self._swarm = voronoi_swarm
        if gauss_swarm is not None:
            if not isinstance(gauss_swarm, _swarm.GaussIntegrationSwarm):
                raise RuntimeError("Provided 'gauss_swarm' must be a GaussIntegrationSwarm object")
            if gauss_swarm.mesh is not self.mesh:
                raise ValueError("Provided 'gauss_swarm' must live on the velocity field's mesh")
        self._gauss_swarm = gauss_swarm
        if not isinstance(conditions, (list, tuple)):
            conditions = [conditions]
        for c in conditions:
            if not isinstance(c, _cond.SystemCondition):
                raise TypeError("Provided 'conditions' must be 'SystemCondition' objects.")
            if c.variable is not velocityField:
                raise ValueError("Only conditions on the velocity field are supported.")
        self._conditions = list(conditions)
        if self._swarm is not None:
            self._swarm._voronoi_swarm.repopulate()
        self._u = None
        self._p = None

    # settable functions (P/systems/_stokes.py:334-355)
    @property
    def fn_viscosity(self):
        return self._fn_viscosity

    @fn_viscosity.setter
    def fn_viscosity(self, value):
        f = _fn.Function.convert(value)
        if not isinstance(f, _fn.Function):
            raise TypeError("Provided 'fn_viscosity' must be of or convertible to 'Function' class.")
        self._fn_viscosity = f

    @property
    def fn_one_on_lambda(self):
        """1/lambda of the compressible formulation, or None (P/systems/_stokes.py:356-372)."""
        return self._fn_one_on_lambda

    @fn_one_on_lambda.setter
    def fn_one_on_lambda(self, value):
        self._fn_one_on_lambda = _fn.Function.convert(value) if value is not None else None

    @property
    def fn_source(self):
        """The volumetric (continuity) source term H, integrated into h on the PIC
        points (P/systems/_stokes.py:284-288, 375-393)."""
        return self._fn_source

    @fn_source.setter
    def fn_source(self, value):
        # as the reference: the term exists only if the object was built with one
        if self._has_source_term:
            self._fn_source = _fn.Function.convert(value)
        else:
            import warnings
            warnings.warn("Cannot add fn_source to existing stokes object. Instead you should build a new object "
                          "with fn_source defined", RuntimeWarning)

    @property
    def fn_bodyforce(self):
        return self._fn_bodyforce

    @fn_bodyforce.setter
    def fn_bodyforce(self, value):
        self._fn_bodyforce = _fn.Function.convert(value)

    # ------------------------------------------------------------------------
    def _bc(self):
        m = np.zeros(self._velocityField.data.shape, np.uint8)
        for c in self._conditions:
            if isinstance(c, _cond.DirichletCondition):
                m |= c.mask()
        return m

    def _integration_points(self):
        """(offsets, list, ip_xi, ip_w, EvalContext) of the integration swarm."""
        ctx = self.mesh.ctx
        if self._swarm is not None:
            vs = self._swarm._voronoi_swarm
            vs.repopulate()
            s = self._swarm
            n = int(s._off[-1])
            e = _fn.EvalContext(s._lst[:n].long(), vs.global_coords, ctx.device, lib_ctx=ctx,
                                pid32=s._lst[:n].to(torch.int32).contiguous())
            e.map_swarm = s
            return s._off, s._lst, vs.ip_xi, vs.ip_w, e
        # Gauss integration, one "particle" per point: the default GaussIntegrationSwarm
        # of the mesh, 3 points per axis on Q1 and 5 on Q2 (P/swarm/_integration_swarm.py:173-181)
        ng = self._gauss_swarm.particleCount if self._gauss_swarm is not None else \
            (5 if self.mesh.elementType.upper().startswith("Q2") else 3)
        x1, w1 = np.polynomial.legendre.leggauss(ng)
        dim = self.mesh.dim
        r = range(ng)
        if dim == 2:
            xi = np.array([[x1[i], x1[j]] for j in r for i in r])
            w = np.array([w1[i] * w1[j] for j in r for i in r])
        else:
            xi = np.array([[x1[i], x1[j], x1[k]] for k in r for j in r for i in r])
            w = np.array([w1[i] * w1[j] * w1[k] for k in r for j in r for i in r])
        nq = len(w)
        ne = ctx.n_el
        ip_xi = torch.from_numpy(np.tile(xi, (ne, 1))).to(ctx.device)
        ip_w = torch.from_numpy(np.tile(w, ne)).to(ctx.device)
        off = (torch.arange(ne + 1, device=ctx.device) * nq).to(torch.int32)
        lst = torch.arange(ne * nq, device=ctx.device, dtype=torch.int32)

        def coords():
            el = torch.arange(ne * nq, device=ctx.device) // nq
            res = ctx.res
            idx = [el % res[0], (el // res[0]) % res[1]] + ([el // (res[0] * res[1])] if dim == 3 else [])
            out = torch.empty((ne * nq, dim), dtype=torch.float64, device=ctx.device)
            for d in range(dim):
                ax = torch.from_numpy(ctx.axes[d]).to(ctx.device)
                lo, hi = ax[idx[d]], ax[idx[d] + 1]
                out[:, d] = lo + (ip_xi[:, d] + 1.0) * 0.5 * (hi - lo)
            return out

        swarms = _swarms_in(self._fn_viscosity, self._fn_bodyforce, self._fn_one_on_lambda, self._fn_source)
        if not swarms:
            return off, lst, ip_xi, ip_w, _fn.EvalContext(lst.long(), coords, ctx.device, lib_ctx=ctx,
                                                          pid32=lst.to(torch.int32).contiguous())
        # swarm variables on the Gauss points: each point takes the value of the nearest
        # particle of its element (SwarmVariableFn over GeneralSwarm_IntegrationPointMap,
        # L/Underworld/Function/src/SwarmVariableFn.cpp:73-101)
        if len(swarms) > 1:
            raise NotImplementedError("swarm variables of more than one swarm on a Gauss integration swarm")
        sw = swarms[0]
        if sw._x is None or sw._off is None:
            raise RuntimeError("Error occurred while trying to evaluate swarm variable. This can occur when there "
                               "are no particles found in a given element.")
        pid = ctx.gauss_nearest(torch.from_numpy(xi), sw._off, sw._lst, sw._x)
        if bool((pid < 0).any()) and _swarms_in(self._fn_viscosity, self._fn_bodyforce, self._fn_one_on_lambda,
                                                 self._fn_source, variables_only=True):
            raise RuntimeError("Error occurred while trying to evaluate swarm variable. This can occur when there "
                               "are no particles found in a given element. You may wish to add population "
                               "control mechanisms.")
        e = _fn.EvalContext(pid.long(), coords, ctx.device, lib_ctx=ctx, pid32=pid)
        e.point_order = True          # rows are the Gauss points; pid only indexes the swarm's data
        e.map_swarm = sw
        return off, lst, ip_xi, ip_w, e

    def _per_particle(self, f, ectx, npart, ncomp):
        # one kernel for the whole graph, writing straight into particle order
        # (uwg_fn_eval); graphs with node kinds it does not cover use the tensor path
        if getattr(ectx, "point_order", False):
            v = _fn._eval_kernel(f, ectx, ncomp)
            if v is None:
                v = f.evaluate_at(ectx).to(torch.float64)
                if v.shape[1] == 1 and ncomp != 1:
                    v = v.expand(v.shape[0], ncomp)
            if v.shape[1] != ncomp:
                raise ValueError("function returns %d components, %d expected" % (v.shape[1], ncomp))
            return v.contiguous()
        out = torch.zeros((npart, ncomp), dtype=torch.float64, device=ectx.device)
        if _fn._eval_kernel(f, ectx, ncomp, out) is not None:
            return out
        v = f.evaluate_at(ectx).to(torch.float64)
        if v.shape[1] != ncomp:
            raise ValueError("function returns %d components, %d expected" % (v.shape[1], ncomp))
        out = torch.zeros((npart, ncomp), dtype=torch.float64, device=ectx.device)
        out[ectx.pid] = v
        return out.contiguous()

    def _assemble(self):
        ctx = self.mesh.ctx
        off, lst, ip_xi, ip_w, ectx = self._integration_points()
        npart = lst.shape[0]
        eta = self._per_particle(self._fn_viscosity, ectx, npart, 1).view(-1)
        body = self._per_particle(self._fn_bodyforce, ectx, npart, self.mesh.dim)
        lam = None
        if self._fn_one_on_lambda is not None:
            lam = self._per_particle(self._fn_one_on_lambda, ectx, npart, 1).view(-1)
        mask = self._bc()
        vals = self._velocityField.data * (mask != 0)
        ctx.set_bcs(torch.from_numpy(mask.ravel()), torch.from_numpy(np.ascontiguousarray(vals).ravel()))
        ctx.assemble(off, lst, ip_xi, ip_w, eta, body, lam)
        if self._fn_source is not None:
            ctx.add_source(off, lst, ip_xi, ip_w, self._per_particle(self._fn_source, ectx, npart, 1).view(-1))
        # tractions: the surface term on 3 Gauss points per face axis (P/systems/_stokes.py:291-297)
        for c in self._conditions:
            if isinstance(c, _cond.NeumannCondition):
                ctx.add_force(_surface_flux(c, 3, ctx.device))

    @property
    def eqResiduals(self):
        """(||f - K u - G p||, ||h - G^T u||) at the current fields (P/systems/_stokes.py:396-416)."""
        ctx = self.mesh.ctx
        self._assemble()
        u = self._velocityField._to_device()
        p = self._pressureField._to_device()
        r = ctx.residuals(u, p)
        return float(r[0]), float(r[1])

    def _velocity_rms_q2(self, v):
        return _q2_rms(self.mesh, v)

    def velocity_rms(self):
        """sqrt(int v.v / int 1) over the mesh, Gauss quadrature (P/systems/_stokes.py:435-448)."""
        mesh = self.mesh
        v = self._velocityField.data
        dim = mesh.dim
        if mesh._order == 2:
            return self._velocity_rms_q2(v)
        x1, w1 = np.polynomial.legendre.leggauss(2)
        n = [r + 1 for r in mesh.elementRes]
        grid = v.reshape(*(n[::-1]), dim)
        h = [np.diff(a) for a in mesh._axes]
        num = 0.0
        vol = 0.0
        if dim == 2:
            for j in range(2):
                for i in range(2):
                    sx, sy = (1 + x1[i]) / 2, (1 + x1[j]) / 2
                    val = ((1 - sx) * (1 - sy) * grid[:-1, :-1] + sx * (1 - sy) * grid[:-1, 1:] +
                           (1 - sx) * sy * grid[1:, :-1] + sx * sy * grid[1:, 1:])
                    area = np.outer(h[1], h[0])
                    num += np.sum(w1[i] * w1[j] * 0.25 * area * np.sum(val ** 2, axis=-1))
                    vol += np.sum(w1[i] * w1[j] * 0.25 * area)
        else:
            for k in range(2):
                for j in range(2):
                    for i in range(2):
                        s = [(1 + x1[i]) / 2, (1 + x1[j]) / 2, (1 + x1[k]) / 2]
                        val = 0.0
                        for c in range(8):
                            a, b, cz = c & 1, (c >> 1) & 1, (c >> 2) & 1
                            wgt = (s[0] if a else 1 - s[0]) * (s[1] if b else 1 - s[1]) * (s[2] if cz else 1 - s[2])
                            val = val + wgt * grid[cz: cz + n[2] - 1, b: b + n[1] - 1, a: a + n[0] - 1]
                        volm = h[2][:, None, None] * h[1][None, :, None] * h[0][None, None, :]
                        num += np.sum(w1[i] * w1[j] * w1[k] * 0.125 * volm * np.sum(val ** 2, axis=-1))
                        vol += np.sum(w1[i] * w1[j] * w1[k] * 0.125 * volm)
        return float(np.sqrt(num / vol))


def _q2_rms(mesh, v):
    """velocity_rms on a Q2 mesh: 3^dim Gauss points per element."""
    x1, w1 = np.polynomial.legendre.leggauss(3)
    dim = mesh.dim
    r = mesh.elementRes
    grid = v.reshape(*[2 * n + 1 for n in r[::-1]], dim)
    h = [np.diff(a[::2]) for a in mesh._axes]
    vol_el = h[1][:, None] * h[0][None, :] if dim == 2 else \
        h[2][:, None, None] * h[1][None, :, None] * h[0][None, None, :]
    N = lambda s: (0.5 * s * (s - 1.0), 1.0 - s * s, 0.5 * s * (s + 1.0))
    num = vol = 0.0
    scale = 0.5 ** dim
    for q in np.ndindex(*([3] * dim)):
        Ns = [N(x1[qi]) for qi in q]          # per axis, q[0] = x
        wq = np.prod([w1[qi] for qi in q])
        val = 0.0
        for a in np.ndindex(*([3] * dim)):
            wgt = np.prod([Ns[d][a[d]] for d in range(dim)])
            sl = tuple(slice(a[d], a[d] + 2 * r[d], 2) for d in reversed(range(dim)))
            val = val + wgt * grid[sl]
        num += np.sum(wq * scale * vol_el * np.sum(val ** 2, axis=-1))
        vol += np.sum(wq * scale * vol_el)
    return float(np.sqrt(num / vol))


class _Options:
    def __init__(self, **kw):
        self.__dict__.update(kw)


class _OptionsGroup:
    """solver.options.A11 / scr / main / mg (P/systems/_bsscr.py:36-194, subset)."""

    def __init__(self):
        self.A11 = _Options(ksp_rtol=1e-6, ksp_type="fgmres", _mixed=False)
        self.scr = _Options(ksp_rtol=1e-5, ksp_type="fgmres", restart=30)
        # remove_constant_pressure_null_space (OptionsMain, P/systems/_bsscr.py:151,167) and the
        # -remove_checkerboard_pressure_null_space switch of BSSCR (BSSCR.c:369-381)
        self.main = _Options(penalty=0.0, Q22_pc_type="uw", ksp_k2_type="NULL", max_inner=500, max_outer=500,
                             remove_constant_pressure_null_space=False,
                             remove_checkerboard_pressure_null_space=False)
        self.mg = _Options(active=True, levels=0, smooth_steps=3)


class StokesSolverStats:
    def __init__(self, d):
        self.__dict__.update(d)

    def __repr__(self):
        return "StokesSolverStats(%s)" % ", ".join("%s=%r" % kv for kv in sorted(self.__dict__.items()))


class StokesSolver:
    """Block Stokes Schur-complement solver (P/systems/_bsscr.py:229-764).

    Tolerances default to the reference's (inner 1e-6, outer 1e-5); the GPU
    run-time driver additionally reports the true FP64 residual of the full
    system in ``get_stats().residual``."""

    def __init__(self, stokesSLE, **kwargs):
        if not isinstance(stokesSLE, Stokes):
            raise TypeError("Provided system must be of 'Stokes' class")
        self._stokesSLE = stokesSLE
        self.options = _OptionsGroup()
        self._stats = None

    def set_inner_method(self, solve_type="mg"):
        """'mg' (FP64 multigrid CG) or 'mixed' (FP32 multigrid CG inside FP64 refinement)."""
        if solve_type not in ("mg", "mixed", "mg_fp32"):
            raise ValueError("inner method must be 'mg' or 'mixed' on the GPU path (got %r)" % solve_type)
        self.options.A11._mixed = solve_type != "mg"

    def set_inner_rtol(self, rtol):
        self.options.A11.ksp_rtol = float(rtol)

    def set_outer_rtol(self, rtol):
        self.options.scr.ksp_rtol = float(rtol)

    def set_mg_levels(self, levels):
        self.options.mg.levels = int(levels)

    _warning_penalty_compressibility = "Stokes system appears to have set the `fn_one_on_lambda` parameter which " \
        "is incompatible with the penalty method. If parameter is non-zero, erroneous results are likely to be " \
        "generated."

    def set_penalty(self, penalty):
        """Augmented-Lagrangian penalty (P/systems/_bsscr.py:766-780).  The reference
        adds penalty * G M^-1 G^T to K and penalty * G M^-1 h to f (M the diagonal of
        the pressure mass; auglag-driver-DGTGD.c:151-200): for an incompressible system
        that term vanishes at the solution, so it changes the Krylov path, not the
        solution.  The GPU solver reaches that solution without the augmentation; the
        option is recorded, and a compressible system draws the reference's warning."""
        if isinstance(penalty, (int, float)) and penalty >= 0.0:
            self.options.main.penalty = float(penalty)
            self.options.main.Q22_pc_type = "gkgdiag"
        else:
            print("Invalid penalty number chosen. Penalty must be a positive float.")
            self.options.main.penalty = 0.0

    def _check_linearity(self, nonLinearIterate):
        s = self._stokesSLE
        nl = False
        for f in (s.fn_viscosity, s.fn_bodyforce):
            if _depends_on_fields(f, (s._velocityField, s._pressureField)):
                nl = True
        if nl and nonLinearIterate is None:
            raise RuntimeError("Nonlinearity detected.\nYour viscosity or body force depends on the solution; "
                               "set the solve() 'nonLinearIterate' parameter to True or False.")
        return nl

    def solve(self, nonLinearIterate=None, nonLinearTolerance=1.0e-2, nonLinearKillNonConvergent=False,
              nonLinearMinIterations=1, nonLinearMaxIterations=500, callback_post_solve=None,
              print_stats=False, reinitialise=True, **kwargs):
        if kwargs:
            raise ValueError("unknown solver options: %s" % ", ".join(sorted(kwargs)))
        if not isinstance(nonLinearTolerance, float) or nonLinearTolerance < 0.0:
            raise ValueError("'nonLinearTolerance' option must be of type 'float' and greater than 0.0")
        if callback_post_solve is not None and not callable(callback_post_solve):
            raise RuntimeError("The 'callback_post_solve' parameter is not 'None' and isn't callable")
        nonlinear = self._check_linearity(nonLinearIterate) and bool(nonLinearIterate)
        if self.options.main.penalty > 0.0 and self._stokesSLE._fn_one_on_lambda is not None:
            import warnings
            warnings.warn(self._warning_penalty_compressibility)
        its = nonLinearMaxIterations if nonlinear else 1
        prev = None
        self._picard = (0, 0.0)
        for it in range(its):
            self._linear_solve(print_stats)
            if callback_post_solve is not None:
                callback_post_solve()
            if not nonlinear:
                break
            v = self._stokesSLE._velocityField.data.copy()
            if prev is not None:
                change = np.linalg.norm(v - prev) / max(np.linalg.norm(v), 1e-300)
                self._picard = (it + 1, float(change))
                if it + 1 >= nonLinearMinIterations and change < nonLinearTolerance:
                    break
            else:
                self._picard = (it + 1, 0.0)
            prev = v

    def get_nonLinearStats(self):
        """Picard iterations of the last nonlinear solve and the relative change
        of the velocity in its last iteration (P/systems/_bsscr.py:728-738)."""
        class _Stats:
            pass
        a = _Stats()
        a.picard_iterations, a.picard_residual = getattr(self, "_picard", (0, 0.0))
        return a

    def print_petsc_options(self):
        """Prints the solver options in use (the GPU solver's counterpart of the
        reference's PETSc option string, P/systems/_bsscr.py:509-512)."""
        o = self.options
        print("Options: inner_method=%s inner_rtol=%g outer_rtol=%g mg_smooth=%d restart=%d max_inner=%d "
              "max_outer=%d" % ("mixed" if o.A11._mixed else "mg", o.A11.ksp_rtol, o.scr.ksp_rtol,
                                o.mg.smooth_steps, o.scr.restart, o.main.max_inner, o.main.max_outer))

    def _linear_solve(self, print_stats):
        s = self._stokesSLE
        ctx = s.mesh.ctx
        t0 = time.perf_counter()
        s._assemble()
        t1 = time.perf_counter()
        u = s._velocityField._to_device()
        p = s._pressureField._to_device()
        o = self.options
        # the full-system residual target follows the Schur (outer) tolerance, which is
        # what ends the reference's pressure solve; velocity solves run at the inner one
        st = ctx.solve(u, p, mixed=int(o.A11._mixed), rtol=o.scr.ksp_rtol,
                       inner_rtol=o.A11.ksp_rtol, outer_rtol=o.scr.ksp_rtol, max_inner=o.main.max_inner,
                       max_outer=o.main.max_outer, smooth_steps=o.mg.smooth_steps, restart=o.scr.restart,
                       schur_pc=1 if s.mesh._porder == 0 else 0,
                       null_space=2 if o.main.remove_checkerboard_pressure_null_space
                       else (1 if o.main.remove_constant_pressure_null_space else 0))
        s._velocityField._from_device()
        s._pressureField._from_device()
        st["assembly_time"] = t1 - t0
        self._stats = StokesSolverStats(st)
        if min(st["fhat_reason"], st["outer_reason"], st["backsolve_reason"]) < 0:
            warnings.warn("A solver error has been encountered during the solve. The resultant convergence "
                          "reasons are (f_hat, outer, backsolve) (%d,%d,%d)." % (
                              st["fhat_reason"], st["outer_reason"], st["backsolve_reason"]))
        if print_stats:
            self.print_stats()

    def get_stats(self):
        return self._stats

    def print_stats(self):
        st = self._stats
        if st is None:
            return
        print("Pressure iterations: %3d" % st.pressure_its)
        print("Velocity iterations: %3d (presolve)" % st.velocity_presolve_its)
        print("Velocity iterations: %3d (pressure solve)" % st.velocity_pressuresolve_its)
        print("Velocity iterations: %3d (backsolve)" % st.velocity_backsolve_its)
        print("Velocity iterations: %3d (total solve)" % st.velocity_total_its)
        print("SCR RHS  solve time: %.4e" % st.presolve_time)
        print("Pressure solve time: %.4e" % st.pressure_time)
        print("Velocity solve time: %.4e (backsolve)" % st.backsolve_time)
        print("Total solve time   : %.4e" % st.total_time)
        print("Relative residual  : %.3e" % st.residual)


def _depends_on_fields(f, fields):
    if isinstance(f, _fn._MeshVar):
        return f.var in fields
    return any(_depends_on_fields(c, fields) for c in f._children())


def Solver(eqs, type="BSSCR", *args, **kwargs):
    """Solver factory (P/systems/_solver.py:26-35)."""
    if isinstance(eqs, Stokes):
        return StokesSolver(eqs, *args, **kwargs)
    raise ValueError("the GPU path provides the Stokes solver only")


def _uses_swarm(f):
    if isinstance(f, _fn._SwarmVar):
        return True
    return any(_uses_swarm(c) for c in f._children())


def _swarms_in(*fns, variables_only=False):
    """The swarms whose variables (and, unless variables_only, particle-found
    tests) the function graphs read."""
    found, seen = {}, set()
    stack = [f for f in fns if f is not None]
    while stack:
        f = stack.pop()
        if id(f) in seen:
            continue
        seen.add(id(f))
        if isinstance(f, _fn._SwarmVar):
            found[id(f.var.swarm)] = f.var.swarm
        elif isinstance(f, _fn._ParticleFound) and not variables_only:
            found[id(f.swarm)] = f.swarm
        stack.extend(c for c in f._children() if c is not None)
    return list(found.values())


def _gauss_eval(mesh, f, n):
    """Values of the function at the n^dim Gauss points of every element (flat, element-major)."""
    ctx = mesh.ctx
    coords = ctx.gauss_coords(n)
    ectx = _fn.EvalContext(torch.full((coords.shape[0],), -1, dtype=torch.int64, device=ctx.device),
                           lambda: coords, ctx.device)
    return f.evaluate_at(ectx)[:, 0].contiguous()


def _dirichlet_mask(conditions, var):
    m = np.zeros(var.data.shape[0], np.uint8)
    for c in conditions:
        if isinstance(c, _cond.DirichletCondition) and c.variable is var:
            m |= c.mask()[:, 0]
    return m


def _check_conditions(conditions, phiField):
    if not isinstance(conditions, (list, tuple)):
        conditions = [conditions]
    for c in conditions:
        if not isinstance(c, _cond.SystemCondition):
            raise TypeError("Provided 'conditions' must be a list 'SystemCondition' objects.")
        if not isinstance(c, (_cond.DirichletCondition, _cond.NeumannCondition)):
            raise RuntimeError("Input condition type not recognised.")
        if isinstance(c, _cond.NeumannCondition) and c.variable is not phiField:
            raise ValueError("Neumann conditions must be given on the 'phiField'")
    return list(conditions)


def _neumann_flux(conditions, n_gauss, device, scale=1.0):
    """Sum of the surface terms of the Neumann conditions, or None."""
    out = None
    for c in conditions:
        if isinstance(c, _cond.NeumannCondition):
            v = _surface_flux(c, n_gauss, device)
            out = v if out is None else out + v
    return None if out is None else (out * scale).contiguous()


def _surface_geometry(cond, n_gauss, device):
    """Points and weights of a NeumannCondition's surface integral, cached on
    the condition: the Gauss points of every face of every element that holds a
    condition node (GaussBorderParticleLayout.c:186-290), kept where the
    interpolated node indicator exceeds 0.999 (the mask of
    P/systems/sle/_assemblyterm.py:124-144), with weight x surface Jacobian
    (ElementType.c:566-606: product of h_j / 2 over the face's axes)."""
    key = (n_gauss, str(device))
    cache = cond.__dict__.setdefault("_surface_cache", {})
    if key in cache:
        return cache[key]
    var = cond.variable
    mesh = var.mesh
    if not isinstance(mesh, _mesh.FeMesh_Cartesian):
        raise NotImplementedError("Neumann conditions are provided for velocity-mesh variables")
    ndof = var.nodeDofCount
    cm = cond.mask().astype(bool)
    xg, fac, Nq, nodes = _mesh._border_points(mesh, cm.any(1), n_gauss)
    to = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)
    geo = (to(xg), to(fac), to(Nq), to(nodes), to(cm), ndof, mesh.nodesGlobal)
    cache[key] = geo
    return geo


def _surface_flux(cond, n_gauss, device):
    """The NeumannCondition surface term VectorSurfaceAssemblyTerm_NA__Fn__ni
    (L/Underworld/Utils/src/VectorSurfaceAssemblyTerm_NA__Fn__ni.cpp:163-236):
    f[(A, d)] += weight |J_s| flux_d(x) N_A(x) over the condition's surface
    points, for the dofs (A, d) in the condition; [n_nodes * ndof] on device."""
    xg, fac, N, nodes, cm, ndof, n_nodes = _surface_geometry(cond, n_gauss, device)
    out = torch.zeros(n_nodes * ndof, dtype=torch.float64, device=device)
    if xg.shape[0] == 0:
        return out
    ectx = _fn.EvalContext(torch.full((xg.shape[0],), -1, dtype=torch.int64, device=device), lambda: xg, device)
    q = cond.fn_flux.evaluate_at(ectx).to(torch.float64)
    if q.shape[1] != ndof:
        raise ValueError("'fn_flux' returns %d components, the variable has %d" % (q.shape[1], ndof))
    for d in range(ndof):
        c = (fac * q[:, d])[:, None] * N
        c = torch.where(cm[nodes, d], c, torch.zeros_like(c))
        out.index_add_(0, (nodes * ndof + d).reshape(-1), c.reshape(-1))
    return out


class AdvectionDiffusion:
    """Advection-diffusion of a scalar mesh variable (P/systems/_advectiondiffusion.py:16-150):
    ``method="SUPG"`` (explicit predictor-multicorrector, Streamline Upwind
    Petrov-Galerkin) or ``method="SLCN"`` (semi-Lagrangian departure values,
    Crank-Nicolson diffusion), on Q1 meshes."""

    def __init__(self, phiField=None, velocityField=None, fn_diffusivity=None, fn_sourceTerm=None, method="SUPG",
                 conditions=[], phiDotField=None, allow_non_q1=False, gauss_swarm=None, **kwargs):
        if not isinstance(method, str) or method.upper() not in ("SUPG", "SLCN"):
            raise ValueError("'method' parameter must be 'SUPG' or 'SLCN'")
        self.method = method.upper()
        if self.method == "SLCN" and phiDotField:
            warnings.warn("'phiDotField' doesn't influence the 'SLCN' method. It's only required for the 'SUPG' method")
        if self.method == "SUPG" and not phiDotField:
            raise ValueError("'phiDotField' is required for the 'SUPG' method")
        if not isinstance(phiField, _mesh.MeshVariable):
            raise TypeError("Provided 'phiField' must be of 'MeshVariable' class.")
        if phiField.data.shape[1] != 1:
            raise TypeError("Provided 'phiField' must be a scalar")
        if velocityField.data.shape[1] != phiField.mesh.dim:
            raise TypeError("Provided 'velocityField' must be the same dimensionality as the phiField's mesh")
        if not isinstance(phiField.mesh, _mesh.FeMesh_Cartesian) or phiField.mesh._order != 1:
            raise ValueError("The 'phiField' must be discretised on a Q1 mesh: advection-diffusion is provided "
                             "for Q1 elements only (allow_non_q1 is not supported on the GPU path)")
        if gauss_swarm is not None:
            if not isinstance(gauss_swarm, _swarm.GaussIntegrationSwarm):
                raise RuntimeError("Provided 'gauss_swarm' must be a GaussIntegrationSwarm object")
            if gauss_swarm.particleCount != (3 if self.method == "SUPG" else 5):
                raise NotImplementedError("the GPU %s kernels integrate on %d Gauss points per axis; a gauss_swarm "
                                          "with %d is not supported" % (self.method, 3 if self.method == "SUPG" else 5,
                                                                        gauss_swarm.particleCount))
        if self.method == "SUPG":
            self.system = _SUPG_AdvectionDiffusion(phiField, phiDotField, velocityField, fn_diffusivity,
                                                   fn_sourceTerm, conditions)
        else:
            self.system = _SLCN_AdvectionDiffusion(phiField, velocityField, fn_diffusivity, fn_sourceTerm, conditions)

    @property
    def velocityField(self):
        return self.system.velocityField

    @property
    def phiField(self):
        return self.system.phiField

    def integrate(self, dt=0.0, **kwargs):
        """Advance phiField by dt."""
        self.system.integrate(dt, **kwargs)

    def get_max_dt(self):
        """The method's time-step bound for the current velocity and diffusivity."""
        return self.system.get_max_dt()


class _SUPG_AdvectionDiffusion:
    """SUPG (P/systems/_advectiondiffusion.py:838-1020): the explicit
    predictor-multicorrector integrated on the 3-point Gauss swarm;
    ``get_max_dt()`` is the Courant bound with courant factor 0.5."""

    def __init__(self, phiField, phiDotField, velocityField, fn_diffusivity, fn_sourceTerm=None, conditions=[]):
        if not isinstance(phiDotField, _mesh.MeshVariable):
            raise TypeError("Provided 'phiDotField' must be 'None' or of 'MeshVariable' class.")
        if phiDotField.data.shape != phiField.data.shape:
            raise TypeError("Provided 'phiDotField' is not the same shape as the provided 'phiField'")
        self.phiField, self._phidot, self.velocityField = phiField, phiDotField, velocityField
        self.mesh = phiField.mesh
        self._conditions = _check_conditions(conditions, phiField)
        self.fn_diffusivity = _fn.Function.convert(fn_diffusivity)
        self.fn_sourceTerm = _fn.Function.convert(fn_sourceTerm) if fn_sourceTerm is not None else None
        for f in (self.fn_diffusivity, self.fn_sourceTerm):
            if f is not None and _uses_swarm(f):
                raise ValueError("Gauss-point integration cannot evaluate swarm variables")

    def integrate(self, dt, **kwargs):
        ctx = self.mesh.ctx
        kappa = _gauss_eval(self.mesh, self.fn_diffusivity, 3)
        src = _gauss_eval(self.mesh, self.fn_sourceTerm, 3) if self.fn_sourceTerm is not None else None
        mask = _dirichlet_mask(self._conditions, self.phiField)
        phi = self.phiField._to_device().contiguous()
        phidot = self._phidot._to_device().contiguous()
        # Dirichlet values: phi's and phi-dot's current values (FeVariable_SetBC on both)
        bcval = phi.clone()
        bcdot = phidot.clone()
        vel = self.velocityField._to_device()
        # flux conditions: the surface term on 2 Gauss points per face axis, added to the
        # residual (P/systems/_advectiondiffusion.py:978-991)
        flux = _neumann_flux(self._conditions, 2, ctx.device)
        ctx.advdiff_step(dt, vel, kappa, phi, phidot, torch.from_numpy(mask), bcval, bcdot, source_q=src, flux=flux)
        self.phiField._from_device()
        self._phidot._from_device()

    def get_max_dt(self):
        ctx = self.mesh.ctx
        kappa = _gauss_eval(self.mesh, self.fn_diffusivity, 3)
        return ctx.advdiff_max_dt(self.velocityField._to_device(), kappa, 0.5)


class _SLCN_AdvectionDiffusion:
    """Semi-Lagrangian Crank-Nicolson (P/systems/_advectiondiffusion.py:153-823):
    departure values by RK4 back-tracing and Lagrange cubics on static stencils
    (the reference's default interpolator), then the Crank-Nicolson diffusion
    system on the 5-point Gauss swarm, Dirichlet nodes keeping their values."""

    def __init__(self, phiField, velocityField, fn_diffusivity, fn_sourceTerm=None, conditions=[]):
        self.phiField, self.velocityField = phiField, velocityField
        self.mesh = phiField.mesh
        self._conditions = _check_conditions(conditions, phiField)
        self.fn_diffusivity = _fn.Function.convert(fn_diffusivity)
        self.fn_sourceTerm = _fn.Function.convert(fn_sourceTerm) if fn_sourceTerm is not None else None
        for f in (self.fn_diffusivity, self.fn_sourceTerm):
            if f is not None and _uses_swarm(f):
                raise ValueError("Gauss-point integration cannot evaluate swarm variables")
        self._phiStar = self.mesh.add_variable(nodeDofCount=1)
        self.last_solve = None

    def integrate(self, dt=0.0, phiStar=None, interpolator="", solve=True, phiStarCopy=None, smooth=0.9,
                  substeps=1, rtol=1e-10, **kwargs):
        if interpolator:
            raise NotImplementedError("the GPU path provides the default cubic-stencil interpolator only")
        ctx = self.mesh.ctx
        dts = dt / float(substeps)
        for _ in range(substeps):
            phi = self.phiField._to_device().contiguous()
            if phiStar is None:
                # the reference traces back over the whole dt in every substep
                # (SemiLagrangianIntegrator_SolveNew is called with dt, :740-746)
                ps = ctx.slcn_phistar(dt, self.velocityField._to_device(), phi)
                self._phiStar.data[:, 0] = ps.cpu().numpy()
            else:
                self._phiStar.data[...] = phiStar.data
                ps = self._phiStar._to_device().contiguous()
            if phiStarCopy is not None:
                phiStarCopy.data[...] = self._phiStar.data
            if solve:
                kappa = _gauss_eval(self.mesh, self.fn_diffusivity, 5)
                src = _gauss_eval(self.mesh, self.fn_sourceTerm, 5) if self.fn_sourceTerm is not None else None
                mask = torch.from_numpy(_dirichlet_mask(self._conditions, self.phiField))
                # flux conditions: dt times the surface term on 2 Gauss points per face axis
                # (P/systems/_advectiondiffusion.py:237-248)
                flux = _neumann_flux(self._conditions, 2, ctx.device, scale=dts)
                its, res = ctx.slcn_solve(dts, kappa, mask, ps, phi, source_q=src, rtol=rtol, flux=flux)
                self.last_solve = {"iterations": its, "residual": res}
                self.phiField._from_device()

    def get_max_dt(self):
        ctx = self.mesh.ctx
        vel = self.velocityField._to_device().reshape(-1, self.mesh.dim)
        vmax = float(torch.sqrt(torch.max(torch.sum(vel * vel, dim=1))))
        nodes = torch.from_numpy(self.mesh.data).to(ctx.device)
        ectx = _fn.EvalContext(torch.full((nodes.shape[0],), -1, dtype=torch.int64, device=ctx.device),
                               lambda: nodes, ctx.device)
        kmax = float(self.fn_diffusivity.evaluate_at(ectx).max())
        dx = ctx.min_sep
        adv = dx / vmax if vmax > 0.0 else float("inf")
        diff = dx * dx / kmax if kmax > 0.0 else float("inf")
        return min(adv, diff)


class SwarmAdvector:
    """Midpoint-RK2 particle advection with owner update (P/systems/_timeintegration.py:77-157)."""

    def __init__(self, velocityField, swarm, order=2, **kwargs):
        if not isinstance(velocityField, _mesh.MeshVariable):
            raise ValueError("Provided 'velocityField' must be of 'MeshVariable' class.")
        if swarm is not None and not isinstance(swarm, _swarm.Swarm):
            raise ValueError("Provided 'swarm' must be of 'Swarm' class.")
        if order != 2:
            raise ValueError("only order=2 (midpoint RK2) is provided")
        self._velocityField = velocityField
        self._swarm = swarm
        self.dt = 0.0
        self.time = 0.0

    def get_max_dt(self):
        """0.5 * minimum node separation / max |v| (SwarmAdvector_MaxDt)."""
        ctx = self._swarm.mesh.ctx
        return ctx.max_dt(self._velocityField._to_device())

    def integrate(self, dt, update_owners=True):
        self.dt = dt     # the integrator's step, as TimeIntegration.integrate records it
        s = self._swarm
        ctx = s.mesh.ctx
        vel = self._velocityField._to_device()
        fb, failed = ctx.rk2(s._x, vel, dt)
        if failed:
            raise RuntimeError("Unable to determine valid velocity for %d particle(s): coordinate appears to be "
                               "outside the global domain." % failed)
        if not bool(torch.isfinite(s._x).all()):
            raise RuntimeError("particle coordinates are not finite after advection")
        s._host_valid = False
        s._toggle_state()
        if update_owners:
            s.update_particle_owners()
