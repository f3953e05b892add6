"""CPU baseline of the PIC Stokes path (TEST/BENCHMARK INFRASTRUCTURE).

Times the oracle -- the reference's algorithms restated in C (uwo.c) plus the
CPU BSSCR solver (uwo_solve.c) -- with OpenMP on all host cores.  The solver
runs the GPU library's algorithm: velocity solves by multigrid-preconditioned
CG (Chebyshev smoother of the workload's degree: 1 for the 3D GRF workload,
2 in the pairings), flexible GMRES on the Schur complement with the
weighted scaled BFBt preconditioner and its pressure multigrid (the CPU port
in uwo_solve.c), FP64 vectors.

Per workload (``CPUBaseline``), set up once at full size, then per step a
bounded sample:

* coincident mapping + DVC weights: a contiguous slice of elements, scaled by
  the element count;
* PIC assembly + solver setup: the full mesh, once (its time is reported);
* Stokes solve: a converged solve where the mesh is small enough to finish in
  seconds; otherwise (seconds per velocity MG-CG iteration on the full mesh) x
  (velocity iterations) + (seconds per pressure-Laplacian CG iteration on the
  full mesh) x (pressure-Laplacian iterations), the iteration counts taken
  from the GPU's plain FP64 solve of the same algorithm and workload
  (``GPU_FP64_ITS``), and labelled so;
* RK2 advection: a sample of particles, scaled; owner update on all.

``pairings()`` runs full converged CPU solves of the smaller workloads with
both Schur preconditioners, for side-by-side comparison with the same GPU
solves.
"""
import ctypes
import os
import time

import numpy as np

import oracle

# Iteration counts of the GPU's plain FP64 solve (weighted BFBt, pressure-
# Laplacian tolerance 3e-2 with pressure-smoother degree 2, velocity-smoother
# degree 1 as the workload's configuration sets) of the 3D 128^3 GRF workload,
# measured by bench.py on a GB300 (its "fp64_solve" entry): 25 outer, 485
# velocity MG-CG, 1676 pressure-Laplacian CG iterations.
GPU_FP64_ITS = {(3, (128, 128, 128)): {"pressure_its": 25, "velocity_total_its": 485, "schur_pc_its": 1676}}

FULL_SOLVE_MAX_EL = 70000
SMOOTH = 2


def _threads():
    return int(os.environ.get("OMP_NUM_THREADS") or os.cpu_count() or 1)


def _material(kind, x, dim):
    import torch
    if kind == "grf":
        import importlib
        bench = importlib.import_module("bench")
        T = bench.grf_T(torch.from_numpy(x)).numpy()
        eta = np.exp(-11.5 * T)
        body = np.zeros_like(x)
        body[:, 2] = 1e6 * T
        return eta, body
    inside = np.sum((x - np.array([0.5, 0.6])) ** 2, axis=1) < 0.01
    eta = np.where(inside, 100.0, 1.0)
    body = np.zeros_like(x)
    body[:, 1] = np.where(inside, -1.0, 0.0)
    return eta, body


def _mask(m):
    nodes = m.node_coords()
    mask = np.zeros((m.n_nodes, m.dim), np.uint8)
    for d in range(m.dim):
        mask[:, d] = np.isclose(nodes[:, d], 0.0) | np.isclose(nodes[:, d], 1.0)
    return mask.ravel()


def _setup(cfg, res):
    dim = cfg["dim"]
    m = oracle.Mesh(dim, 1, res, (0.0,) * dim, (1.0,) * dim)
    x, _ = m.layout_random(cfg["ppc"], 13)
    eta, body = _material(cfg["kind"], x, dim)
    return m, x, eta, body


def _grow(tbl, cnt, cap=64):
    t = np.full((tbl.shape[0], cap), -1, np.int32)
    t[:, : tbl.shape[1]] = tbl
    return t


def solve_full(cfg, res, schur_pc):
    """A converged CPU solve (to a 1e-8 relative residual) of the workload on `res`."""
    m, x, eta, body = _setup(cfg, res)
    tbl, cnt, _ = m.initial_tables(cfg["ppc"], cfg["ppc"])
    ip_xi, ip_w = m.pic_map(x, tbl, cnt)
    s = oracle.StokesCPU(m)
    s.set_bc(_mask(m))
    s.set_schur_pc(schur_pc, SMOOTH)
    off = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int32)
    lst = tbl.ravel().astype(np.int32)
    t0 = time.perf_counter()
    s.assemble(off, lst, ip_xi[lst], ip_w[lst], eta, body)
    t_asm = time.perf_counter() - t0
    t0 = time.perf_counter()
    u, p, st = s.solve(inner_rtol=1e-10, outer_rtol=1e-9, max_outer=2000, deg=SMOOTH)
    st.update(solve_s=time.perf_counter() - t0, assemble_s=t_asm)
    return st


class CPUBaseline:
    """The CPU port on one workload, set up once; `step()` times one bounded sample."""

    def __init__(self, cfg, workload):
        if cfg.get("order", 1) != 1:
            raise NotImplementedError("the CPU solver port covers Q1/dQ0 only")
        self.cfg, self.workload = cfg, workload
        dim, ppc, res = cfg["dim"], cfg["ppc"], tuple(cfg["res"])
        self.res = res
        t_all = time.perf_counter()
        self.m, self.x, eta, body = _setup(cfg, res)
        m = self.m
        self.n_el, self.npart = m.n_el, len(self.x)
        self.tbl, self.cnt, self.owner = m.initial_tables(ppc, ppc)
        self.frac = 1.0 if self.n_el <= 8192 else 1.0 / 256
        self.n_s = max(1, int(self.n_el * self.frac))
        self.ip_xi = np.zeros((self.npart, dim))
        self.ip_w = np.zeros(self.npart)
        self._map(0, self.n_el)
        self.s = oracle.StokesCPU(m)
        self.s.set_bc(_mask(m))
        self.s.set_schur_pc(1, SMOOTH)
        off = np.concatenate([[0], np.cumsum(self.cnt)]).astype(np.int32)
        lst = self.tbl.ravel().astype(np.int32)
        t0 = time.perf_counter()
        self.s.assemble(off, lst, self.ip_xi[lst], self.ip_w[lst], eta, body)
        self.t_asm = time.perf_counter() - t0
        self.full = None
        if self.n_el <= FULL_SOLVE_MAX_EL:
            t0 = time.perf_counter()
            u, p, st = self.s.solve(inner_rtol=1e-10, outer_rtol=1e-9, max_outer=2000, deg=self.cfg.get("smooth", SMOOTH))
            st["solve_s"] = time.perf_counter() - t0
            self.full = st
        elif (dim, res) not in GPU_FP64_ITS:
            raise NotImplementedError("no GPU iteration counts recorded for %s" % (res,))
        self.vel = np.zeros(m.n_nodes * dim)
        self.vel[::dim] = 1e-3
        self.n_p = self.npart if self.npart <= 2_000_000 else self.npart // 16
        self.setup_s = time.perf_counter() - t_all

    def _map(self, e0, e1):
        p = lambda a: ctypes.c_void_p(a.ctypes.data)
        m = self.m
        oracle.lib().uwo_pic_map(ctypes.byref(m._c), *m._ax(), p(self.x), p(self.tbl), p(self.cnt),
                                 self.tbl.shape[1], e0, e1, 15, p(self.ip_xi), p(self.ip_w))

    def step(self):
        """One bounded sample: mapping + DVC on a slice, one velocity and two
        pressure-Laplacian iterations on the full mesh, RK2 on a sample."""
        t0 = time.perf_counter()
        self._map(0, self.n_s)
        t_map = (time.perf_counter() - t0) * self.n_el / self.n_s
        tv, tl = self.s.time_iterations(1, 2, self.cfg.get("smooth", SMOOTH))
        xs = self.x[: self.n_p].copy()
        t0 = time.perf_counter()
        self.m.rk2(self.vel, 0.1 / max(self.res), xs)
        t_rk2 = (time.perf_counter() - t0) * self.npart / self.n_p
        return {"map_dvc": t_map, "t_vel_it": tv, "t_l_it": tl, "rk2": t_rk2}

    def result(self, samples):
        med = {k: float(np.median([s[k] for s in samples])) for k in samples[0]}
        dim = self.cfg["dim"]
        if self.full is not None:
            t_solve = self.full["solve_s"]
            its = {k: v for k, v in self.full.items() if k not in ("rc", "solve_s")}
            note = "full converged CPU solve"
        else:
            its = GPU_FP64_ITS[(dim, self.res)]
            t_solve = med["t_vel_it"] * its["velocity_total_its"] + med["t_l_it"] * its["schur_pc_its"]
            note = ("solve EXTRAPOLATED: %.3f s per velocity MG-CG iteration and %.4f s per pressure-Laplacian CG "
                    "iteration, measured on the full mesh, x the %d and %d iterations of the GPU's plain FP64 "
                    "solve of the same algorithm (weighted BFBt) and workload"
                    % (med["t_vel_it"], med["t_l_it"], its["velocity_total_its"], its["schur_pc_its"]))
        # owner update of all particles after the sampled RK2 move
        x2 = self.x.copy()
        xs = self.x[: self.n_p].copy()
        self.m.rk2(self.vel, 0.1 / max(self.res), xs)
        x2[: self.n_p] = xs
        t0 = time.perf_counter()
        self.m.update_owners(x2, self.owner.copy(), _grow(self.tbl, self.cnt), self.cnt.copy())
        t_mig = time.perf_counter() - t0
        total = med["map_dvc"] + self.t_asm + t_solve
        return {
            "kind": "port", "cores": _threads(), "workload": self.workload,
            "value": total, "unit": "s/solve",
            "particles_per_s": self.npart / (med["rk2"] + t_mig),
            "phases_s": {"map_dvc": med["map_dvc"], "assemble": self.t_asm, "solve": t_solve, "rk2": med["rk2"],
                         "migrate": t_mig},
            "per_iteration_s": {"velocity_mg_cg": med["t_vel_it"], "pressure_laplacian_cg": med["t_l_it"]},
            "solver_its": its,
            "schur_pc": "weighted scaled BFBt (the GPU library's algorithm, CPU port)",
            "sample": ("map+DVC on %d of %d elements (scaled); assembly and solver setup on the full mesh; %s; "
                       "RK2 on %d of %d particles (scaled), owner update on all" %
                       (self.n_s, self.n_el, note, self.n_p, self.npart)),
            "setup_s": self.setup_s,
        }


def pairings(configs):
    """Full converged CPU solves for side-by-side comparison: the 2D 64^2 sinker with
    both Schur preconditioners and the 3D GRF workload on a 32^3 mesh with BFBt."""
    out = {}
    s2 = dict(configs["sinker2d"])
    for pc, name in ((1, "bfbt"), (0, "uzawa")):
        st = solve_full(s2, tuple(s2["res"]), pc)
        out["sinker2d_64x64_%s" % name] = _brief(st)
    g = dict(configs["grf3d"])
    st = solve_full(g, (32, 32, 32), 1)
    out["grf3d_32x32x32_bfbt"] = _brief(st)
    return out


def _brief(st):
    return {"solve_s": st["solve_s"], "assemble_s": st.get("assemble_s"), "pressure_its": st["pressure_its"],
            "velocity_total_its": st["velocity_presolve_its"] + st["velocity_pressuresolve_its"] +
            st["velocity_backsolve_its"], "schur_pc_its": st.get("schur_pc_its", 0), "residual": st["residual"]}


def measure(cfg, workload, steps=1):
    """Set up and time `steps` samples (the bench's cpu_baseline entry)."""
    b = CPUBaseline(cfg, workload)
    return b.result([b.step() for _ in range(max(1, steps))])
