"""CPU baseline of the PIC Stokes path (TEST/BENCHMARK INFRASTRUCTURE).

Times the oracle -- the reference's algorithms restated in C (uwo.c) plus the
CPU BSSCR solver (uwo_solve.c) -- with OpenMP on all host cores, on a bounded
sample of the benchmark workload, and extrapolates to the full size:

* coincident mapping + DVC weights: a contiguous sample of elements, scaled
  by the element count;
* PIC assembly and owner update: the full workload;
* Stokes solve: (CPU time of one multigrid-preconditioned CG iteration on the
  full mesh) x (inner iterations of the same BSSCR algorithm run to the same
  tolerance on an 8^d mesh of the same workload).  The outer iteration count
  of the reference's Schur preconditioner grows with the resolution, so this
  figure is a lower bound of the full-size CPU solve and is labelled so;
* RK2 advection: a sample of particles, scaled by the particle count.

Every extrapolated figure is labelled in the returned dict.
"""
import os
import time

import numpy as np

import oracle


def _threads():
    return int(os.environ.get("OMP_NUM_THREADS") or os.cpu_count() or 1)


def _material(kind, x, dim):
    import torch
    sys_path_bench = None
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


def _solve_counts(cfg, res):
    """Converged CPU BSSCR on a coarser mesh: iteration counts."""
    m, x, eta, body = _setup(cfg, res)
    tbl, cnt, _ = m.initial_tables(cfg["ppc"], cfg["ppc"])
    ip_xi, ip_w = m.pic_map(x, tbl, cnt)
    s = oracle.StokesCPU(m)
    s.set_bc(_mask(m))
    off = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int32)
    lst = tbl.ravel().astype(np.int32)
    s.assemble(off, lst, ip_xi[lst], ip_w[lst], eta, body)
    t0 = time.perf_counter()
    u, p, st = s.solve(inner_rtol=1e-10, outer_rtol=1e-9)
    st["seconds"] = time.perf_counter() - t0
    return st


def measure(cfg, workload, quick=False):
    if cfg.get("order", 1) != 1:
        raise NotImplementedError("the CPU solver port covers Q1/dQ0 only")
    dim, ppc = cfg["dim"], cfg["ppc"]
    res = cfg["res"]
    L = oracle.lib()
    out = {"kind": "port", "cores": _threads(), "workload": workload}
    t_all = time.perf_counter()
    m, x, eta, body = _setup(cfg, res)
    n_el, npart = m.n_el, len(x)
    tbl, cnt, owner = m.initial_tables(ppc, ppc)

    # 1. mapping + DVC on a sample of elements
    frac = 1.0 if n_el <= 8192 else 1.0 / 256
    n_s = max(1, int(n_el * frac))
    ip_xi = np.zeros((npart, dim))
    ip_w = np.zeros(npart)
    import ctypes
    p = lambda a: ctypes.c_void_p(a.ctypes.data)
    t0 = time.perf_counter()
    L.uwo_pic_map(ctypes.byref(m._c), *m._ax(), p(x), p(tbl), p(cnt), tbl.shape[1], 0, n_s, 15, p(ip_xi), p(ip_w))
    t_map = (time.perf_counter() - t0) * n_el / n_s
    if n_s < n_el:   # the rest of the weights for assembly (untimed)
        L.uwo_pic_map(ctypes.byref(m._c), *m._ax(), p(x), p(tbl), p(cnt), tbl.shape[1], n_s, n_el, 15,
                      p(ip_xi), p(ip_w))

    # 2. assembly + solver setup on the full mesh
    s = oracle.StokesCPU(m)
    s.set_bc(_mask(m))
    off = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int32)
    lst = tbl.ravel().astype(np.int32)
    xi_s, w_s = ip_xi[lst], ip_w[lst]
    t0 = time.perf_counter()
    s.assemble(off, lst, xi_s, w_s, eta, body)
    t_asm = time.perf_counter() - t0

    # 3. solve: per-iteration cost on the full mesh x converged iteration count
    if n_el <= 70000:
        t0 = time.perf_counter()
        u, pr, st = s.solve(inner_rtol=1e-10, outer_rtol=1e-9)
        t_solve = time.perf_counter() - t0
        solve_note = "full converged solve"
        its = st
    else:
        coarse = tuple(min(8, r) for r in res)
        its = _solve_counts(cfg, coarse)
        n_it = its["velocity_presolve_its"] + its["velocity_pressuresolve_its"] + its["velocity_backsolve_its"]
        t0 = time.perf_counter()
        u, pr, st = s.solve(inner_rtol=1e-10, outer_rtol=1e-9, max_inner=3, max_outer=1)
        dt = time.perf_counter() - t0
        it_done = st["velocity_presolve_its"] + st["velocity_pressuresolve_its"] + st["velocity_backsolve_its"]
        t_it = dt / max(it_done, 1)
        t_solve = n_it * t_it
        conv = "converged" if its.get("rc", 0) == 0 else "iteration-capped"
        solve_note = ("solve extrapolated as a LOWER BOUND: %.3f s per MG-CG iteration on the full mesh x %d "
                      "iterations of the %s %s solve (outer iterations of this preconditioner grow with "
                      "resolution)" % (t_it, n_it, conv, "x".join(map(str, coarse))))

    # 4. RK2 on a sample of particles + owner update on all
    vel = np.zeros(m.n_nodes * dim)
    vel[::dim] = 1e-3
    n_p = npart if npart <= 2_000_000 else npart // 16
    xs = x[:n_p].copy()
    t0 = time.perf_counter()
    m.rk2(vel, 0.1 / max(res), xs)
    t_rk2 = (time.perf_counter() - t0) * npart / n_p
    x2 = x.copy()
    x2[:n_p] = xs
    t0 = time.perf_counter()
    m.update_owners(x2, owner, _grow(tbl, cnt), cnt)
    t_mig = time.perf_counter() - t0

    total = t_map + t_asm + t_solve
    out.update({
        "value": total,
        "unit": "s/solve",
        "particles_per_s": npart / (t_rk2 + t_mig),
        "phases_s": {"map_dvc": t_map, "assemble": t_asm, "solve": t_solve, "rk2": t_rk2, "migrate": t_mig},
        "sample": ("map+DVC on %d of %d elements (scaled); assembly and owner update on all %d particles; %s; "
                   "RK2 on %d of %d particles (scaled)" % (n_s, n_el, npart, solve_note, n_p, npart)),
        "solver_its": {k: v for k, v in its.items() if k != "rc"},
        "wall_s": time.perf_counter() - t_all,
    })
    return out


def _grow(tbl, cnt, cap=64):
    t = np.full((tbl.shape[0], cap), -1, np.int32)
    t[:, : tbl.shape[1]] = tbl
    return t
