"""Benchmark of the PIC Stokes path: Stokes solve time to a 1e-8 relative
residual and particles advected per second.

Workload (default ``grf3d``): 3D unit cube, 128^3 Q1/dQ0 elements, free-slip
walls, 20 particles per element (41,943,040 particles) from the seeded
per-cell random layout.  T is a seeded Gaussian random field (correlation
length 0.1, spectral synthesis on a 256^3 grid, Gaussian covariance),
trilinearly sampled at the particles and scaled to [0, 1]; viscosity
exp(-11.5 T) (contrast ~1e5), body force (0, 0, Ra T) with Ra = 1e6.
``sinker2d`` is the 2D 64^2 sinker (circle r=0.1 at (0.5,0.6), viscosity 100,
density 1, gravity (0,-1)) that the reference runs on a CPU.  ``rt2d_q2`` is
the 2D 256^2 Q2/dPc1 Rayleigh-Taylor case: a dense layer (density 1,
viscosity 1) over a light one (density 0, viscosity 0.01) with the interface
at y = 0.2 + 0.02 cos(pi x), per-particle viscosity times a seeded
log-uniform factor in [1e-1, 1e1], 40 particles per element; its Schur
preconditioner is the reference's Uzawa term.

One step = the hot path over the swarm: coincident mapping + DVC weights,
PIC assembly, BSSCR solve to 1e-8 (FP32 inner solves in FP64 refinement; the
plain FP64 solve is timed beside it), RK2 advection at the maximum stable dt,
owner update.  ``value`` = seconds per Stokes solve (mapping + weights +
assembly + solve) with inputs resident on the device; ``e2e`` = the same
measured through host buffers (particle coordinates, viscosity and body
force copied in, velocity and pressure copied out, every step).

``--impl reference`` times the CPU oracle (the reference's algorithms
restated in C, OpenMP on all host cores) on a bounded sample of the same
workload, extrapolated to the full size and labelled as such.
"""
import argparse
import json
import re
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    # smooth: Chebyshev degree of the velocity multigrid smoother (degree 1 is the
    # fastest on the GRF workload: more but cheaper MG-CG iterations)
    "grf3d": dict(dim=3, res=(128, 128, 128), ppc=20, kind="grf", smooth=1),
    "grf3d_small": dict(dim=3, res=(32, 32, 32), ppc=20, kind="grf", smooth=1),
    "sinker2d": dict(dim=2, res=(64, 64), ppc=20, kind="sinker"),
    # 2D Q2/dPc1 Rayleigh-Taylor layering, 40 particles per element
    "rt2d_q2": dict(dim=2, res=(256, 256), ppc=40, kind="rt", order=2, porder=1),
    # 3D Q2/dPc1 thermal-convection Stokes step: T = 1 - z + seeded 1e-2 noise,
    # viscosity exp(-9.2 T), buoyancy Ra T (Ra = 1e6), 30 particles per element
    "conv3d_q2": dict(dim=3, res=(96, 96, 96), ppc=30, kind="conv", order=2, porder=1),
    "conv3d_q2_small": dict(dim=3, res=(32, 32, 32), ppc=30, kind="conv", order=2, porder=1),
}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {"hbm_gbs": 6800.0, "_fallback": True}


# ---------------------------------------------------------------------------
# synthetic inputs
# ---------------------------------------------------------------------------
def grf_T(x, seed=1234, n=256, corr=0.1):
    """Seeded Gaussian random field (Gaussian covariance, length corr) on an
    n^3 periodic grid over the unit cube, trilinearly sampled at x, min-max
    scaled to [0, 1].  Input generation only (torch)."""
    import torch
    g = torch.Generator(device=x.device).manual_seed(seed)
    noise = torch.randn((n, n, n), generator=g, device=x.device, dtype=torch.float32)
    k = torch.fft.fftfreq(n, d=1.0 / n, device=x.device).float() * 2 * torch.pi
    k2 = k[:, None, None] ** 2 + k[None, :, None] ** 2 + k[None, None, :] ** 2
    amp = torch.exp(-k2 * corr * corr / 4.0)          # sqrt of the Gaussian spectrum
    f = torch.fft.ifftn(torch.fft.fftn(noise) * amp).real
    f = (f - f.min()) / (f.max() - f.min())
    # trilinear sample (grid point i at i/(n-1))
    u = x.float() * (n - 1)
    i0 = u.floor().clamp(0, n - 2).long()
    t = (u - i0.float()).clamp(0, 1)
    out = torch.zeros(x.shape[0], device=x.device, dtype=torch.float32)
    for c in range(8):
        a, b, cc = c & 1, (c >> 1) & 1, (c >> 2) & 1
        w = ((t[:, 0] if a else 1 - t[:, 0]) * (t[:, 1] if b else 1 - t[:, 1]) * (t[:, 2] if cc else 1 - t[:, 2]))
        out += w * f[i0[:, 2] + cc, i0[:, 1] + b, i0[:, 0] + a]
    T = out.double()
    return (T - T.min()) / (T.max() - T.min())


def material(cfg, x):
    import torch
    dim = cfg["dim"]
    if cfg["kind"] == "grf":
        T = grf_T(x)
        eta = torch.exp(-11.5 * T)
        body = torch.zeros_like(x)
        body[:, 2] = 1e6 * T
        return eta.contiguous(), body.contiguous()
    if cfg["kind"] == "conv":
        # seeded smooth perturbation: a few random Fourier modes vanishing at z = 0, 1
        g = torch.Generator(device="cpu").manual_seed(4242)
        a = (torch.rand(4, 3, generator=g, dtype=torch.float64) * 2.0 - 1.0).tolist()
        noise = torch.zeros(x.shape[0], dtype=torch.float64, device=x.device)
        for k in range(1, 5):
            ax, ay, az = a[k - 1]
            noise += ax * torch.cos(torch.pi * k * x[:, 0] + ay) * torch.cos(torch.pi * k * x[:, 1] + az) * \
                torch.sin(torch.pi * x[:, 2])
        T = (1.0 - x[:, 2] + 0.01 * noise / 4.0).clamp(0.0, 1.0)
        eta = torch.exp(-9.2 * T)
        body = torch.zeros_like(x)
        body[:, 2] = 1e6 * T
        return eta.contiguous(), body.contiguous()
    if cfg["kind"] == "rt":
        g = torch.Generator(device=x.device).manual_seed(4321)
        dense = x[:, 1] > 0.2 + 0.02 * torch.cos(torch.pi * x[:, 0])
        fac = 10.0 ** (2.0 * torch.rand(x.shape[0], generator=g, device=x.device, dtype=torch.float64) - 1.0)
        eta = torch.where(dense, 1.0, 0.01).double() * fac
        body = torch.zeros_like(x)
        body[:, 1] = torch.where(dense, -1.0, 0.0)
        return eta.contiguous(), body.contiguous()
    inside = ((x - torch.tensor([0.5, 0.6], device=x.device, dtype=x.dtype)) ** 2).sum(1) < 0.01
    eta = torch.where(inside, 100.0, 1.0).double()
    body = torch.zeros_like(x)
    body[:, 1] = torch.where(inside, -1.0, 0.0)
    return eta.contiguous(), body.contiguous()


def freeslip_mask(ctx):
    import numpy as np
    import torch
    dim = ctx.dim
    n = [r * ctx.order + 1 for r in ctx.res]
    idx = np.arange(int(np.prod(n)))
    ijk = [idx % n[0], (idx // n[0]) % n[1]] + ([idx // (n[0] * n[1])] if dim == 3 else [])
    m = np.zeros((len(idx), dim), np.uint8)
    for d in range(dim):
        m[:, d] = (ijk[d] == 0) | (ijk[d] == n[d] - 1)
    return torch.from_numpy(m.ravel())


# ---------------------------------------------------------------------------
# clocks sampler
# ---------------------------------------------------------------------------
class Clocks:
    def __init__(self):
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        def run():
            q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            while not self._stop.is_set():
                try:
                    out = subprocess.run(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits", "-i", "0"],
                                         capture_output=True, text=True, timeout=5).stdout.strip()
                    self.samples.append([s.strip() for s in out.split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)
        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)
        mhz = sorted(float(s[0]) for s in self.samples if s and s[0].replace(".", "").isdigit())
        mx = next((float(s[1]) for s in self.samples if len(s) > 1 and s[1].replace(".", "").isdigit()), None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 2 + i and s[2 + i].lower() == "active"})
        return {"sm_mhz": mhz[len(mhz) // 2] if mhz else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(self.samples)}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_gpu(args):
    import numpy as np
    import torch
    from underworld2_gb300._core import Context, rng_seed

    cfg = CONFIGS[args.config]
    dim = cfg["dim"]
    ctx = Context(dim, cfg["res"], (0.0,) * dim, (1.0,) * dim, order=cfg.get("order", 1), porder=cfg.get("porder", 0))
    ctx.set_bcs(freeslip_mask(ctx))
    x0, owner0, off0, lst0, _ = ctx.layout_random(cfg["ppc"], rng_seed(13))
    eta0, body0 = material(cfg, x0)
    npart = x0.shape[0]
    u = ctx.zeros(ctx.n_vdof)
    p = ctx.zeros(ctx.n_pdof)
    opts = dict(rtol=1e-8, inner_rtol=args.inner_rtol, outer_rtol=args.outer_rtol, smooth_steps=cfg.get("smooth", 2), restart=120,
                schur_pc=args.schur_pc if cfg.get("porder", 0) == 0 else 0, schur_pc_rtol=args.bfbt_rtol, schur_pc_its=args.bfbt_its, max_outer=args.max_outer)
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def solve_step(x, off, lst, eta, body, mixed, times):
        e = [ev() for _ in range(4)]
        e[0].record()
        ip_xi = ctx.pic_map(x, off, lst)
        ip_w = ctx.dvc_weights(off, ip_xi)
        e[1].record()
        ctx.assemble(off, lst, ip_xi, ip_w, eta, body)
        e[2].record()
        u.zero_()
        p.zero_()
        st = ctx.solve(u, p, mixed=mixed, **opts)
        e[3].record()
        torch.cuda.synchronize()
        times["map_dvc"].append(e[0].elapsed_time(e[1]) / 1e3)
        times["assemble"].append(e[1].elapsed_time(e[2]) / 1e3)
        times["solve"].append(e[2].elapsed_time(e[3]) / 1e3)
        return st

    def advect(n_steps, times):
        """Successive RK2 steps at the maximum stable dt with the owner update
        (migration between elements) after each, particles stored in FP32 with the
        arithmetic in FP64, from the reset swarm through the solved velocity field."""
        x32 = x0.to(torch.float32)
        own, of, ls = owner0.clone(), off0.clone(), lst0.clone()
        torch.cuda.synchronize()
        for _ in range(n_steps):
            e = [ev() for _ in range(3)]
            e[0].record()
            dt = ctx.max_dt(u)
            ctx.rk2(x32, u, dt)
            e[1].record()
            ctx.update_owners(x32, own, of, ls)
            e[2].record()
            torch.cuda.synchronize()
            times["rk2"].append(e[0].elapsed_time(e[1]) / 1e3)
            times["migrate"].append(e[1].elapsed_time(e[2]) / 1e3)
        moved = int((own != owner0).sum())
        del x32
        return moved

    mixed = 0 if args.mode == "fp64" else 1
    # state copies so every step starts from the same swarm
    x, owner, off, lst = x0.clone(), owner0.clone(), off0.clone(), lst0.clone()
    warm = {k: [] for k in ("map_dvc", "assemble", "solve", "rk2", "migrate")}
    for _ in range(args.warmup):
        x.copy_(x0); owner.copy_(owner0); off.copy_(off0); lst.copy_(lst0)
        solve_step(x, off, lst, eta0, body0, mixed, warm)
    advect(3, warm)

    clocks = Clocks()
    clocks.start()
    times = {k: [] for k in ("map_dvc", "assemble", "solve", "rk2", "migrate")}
    stats = []
    torch.cuda.synchronize()
    for _ in range(args.steps):
        x.copy_(x0); owner.copy_(owner0); off.copy_(off0); lst.copy_(lst0)
        torch.cuda.synchronize()
        stats.append(solve_step(x, off, lst, eta0, body0, mixed, times))
    torch.cuda.synchronize()
    # advection of the workload: ten successive steps (FP32 storage, FP64 arithmetic)
    moved = advect(10, times)
    clk = clocks.stop()

    # plain FP64 solve on the same assembled system (one timed run); the error of the
    # mixed-precision solution against it (pressure modulo its constant null mode)
    u_mix, p_mix = u.clone(), p.clone()
    fp64 = None
    if not args.skip_fp64 and mixed:
        x.copy_(x0); owner.copy_(owner0); off.copy_(off0); lst.copy_(lst0)
        t64 = {k: [] for k in ("map_dvc", "assemble", "solve")}
        st64 = solve_step(x, off, lst, eta0, body0, 0, t64)
        pm, p64 = p_mix - p_mix.mean(), p - p.mean()
        fp64 = {"solve_s": t64["solve"][0], "pressure_its": st64["pressure_its"],
                "velocity_total_its": st64["velocity_total_its"], "schur_pc_its": st64["schur_pc_its"],
                "residual": st64["residual"],
                "mixed_vs_fp64": {"velocity": float(torch.linalg.norm(u_mix - u) / torch.linalg.norm(u)),
                                  "pressure": float(torch.linalg.norm(pm - p64) / torch.linalg.norm(p64))}}

    # end to end through the drop-in API from numpy host arrays, every step
    e2e = e2e_api(args, cfg, x0.cpu().numpy(), eta0.cpu().numpy(), body0.cpu().numpy(), mixed)
    del u_mix, p_mix

    # roofline of the dominant kernel class: the matrix-free K apply (FP32)
    kinfo = time_kernel_apply(ctx)
    pk = peaks()
    achieved = kinfo["bytes"] / kinfo["seconds"] / 1e9
    per_step = [times["map_dvc"][i] + times["assemble"][i] + times["solve"][i] for i in range(args.steps)]
    solve_s = float(np.mean(per_step))
    adv_s = float(np.mean([times["rk2"][i] + times["migrate"][i] for i in range(len(times["rk2"]))]))
    line = {
        "metric": "Stokes solve time @1e-8 resid (learned+FP32 vs FP64 GPU); particles/s advected",
        "value": solve_s,
        "unit": "s/solve",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * solve_s,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if not mixed else "f32+f64",
        "data": "synthetic",
        "config": workload_config(args.config, npart),
        "solve_mode": args.mode,
        "particles_per_s": npart / adv_s,
        "advection": {"steps": 10, "storage": "FP32 coordinates, FP64 arithmetic", "s_per_step": adv_s,
                      "particles_changed_element": moved},
        "throughput": {"K_apply_mdof_per_s": ctx.n_vdof / kinfo["seconds"] / 1e6,
                       "stokes_solves_per_s": 1.0 / solve_s},
        "phases_s": {k: float(np.mean(v)) for k, v in times.items()},
        "solver": {"pressure_its": stats[-1]["pressure_its"], "velocity_total_its": stats[-1]["velocity_total_its"],
                   "schur_pc_its": stats[-1]["schur_pc_its"], "refinement_steps": stats[-1]["refinement_steps"],
                   "residual": stats[-1]["residual"], "schur_pc": "scaled BFBt" if (args.schur_pc and cfg.get("porder", 0) == 0) else "Uzawa S^",
                   "presolve_s": stats[-1]["presolve_time"], "pressure_s": stats[-1]["pressure_time"],
                   "backsolve_s": stats[-1]["backsolve_time"], "schur_pc_s": stats[-1]["schur_pc_time"],
                   "schur_op_s": stats[-1]["schur_op_time"]},
        "fp64_solve": fp64,
        "e2e": e2e,
        "roofline": {"bound": "hbm", "kernel": kinfo["name"], "achieved": achieved, "peak": pk.get("hbm_gbs"),
                     "unit": "GB/s", "frac": achieved / pk.get("hbm_gbs", 6800.0),
                     "peak_source": "fallback" if pk.get("_fallback") else "measured",
                     "traffic": dram_traffic(kinfo["name"], args.config), "bytes_per_launch": kinfo["bytes"],
                     "launch_s": kinfo["seconds"]},
        "clocks": clk,
    }
    if args.count_launches:
        n_solve, n_adv = count_launches(ctx, x0, owner0, off0, lst0, eta0, body0, mixed, opts, u, p)
        line["gpu_launches"] = n_solve * args.steps + n_adv * 10
    line["pairings"] = gpu_pairings()
    if args.cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args)
    return line


def workload_name(key):
    return {"grf3d": "3D 128^3 Q1/dQ0 GRF viscosity exp(-11.5T), Ra=1e6, 20 ppc, free-slip (config 3)",
            "grf3d_small": "3D 32^3 Q1/dQ0 GRF viscosity, 20 ppc, free-slip",
            "sinker2d": "2D 64^2 Q1/dQ0 sinker, 20 ppc, free-slip (config 1)",
            "rt2d_q2": "2D 256^2 Q2/dPc1 Rayleigh-Taylor, 40 ppc, viscosity x 10^U(-1,1), free-slip (config 2)",
            "conv3d_q2": "3D 96^3 Q2/dPc1 convection Stokes step, T = 1 - z + 1e-2 noise, viscosity exp(-9.2T), Ra=1e6, 30 ppc, free-slip (config 5 solve)",
            "conv3d_q2_small": "3D 32^3 Q2/dPc1 convection Stokes step, 30 ppc"}[key]


def workload_config(key, npart=None):
    """The `config` object of both arms' lines (identical keys and values)."""
    import numpy as np
    cfg = CONFIGS[key]
    dim = cfg["dim"]
    if npart is None:
        npart = int(np.prod(cfg["res"])) * cfg["ppc"]
    return {"workload": workload_name(key),
            "mesh": "x".join(map(str, cfg["res"])) + (" Q2/dPc1" if cfg.get("order", 1) == 2 else " Q1/dQ0"),
            "particles": int(npart), "particles_per_cell": cfg["ppc"],
            "inputs_vs_L2": "particle arrays (%.1f GB) exceed the 129 MB L2" % (npart * 8 * (2 * dim + 1) / 1e9)}


def e2e_api(args, cfg, x_h, eta_h, body_h, mixed):
    """The same step through the drop-in API (uw.mesh / uw.swarm / uw.systems) from
    numpy host arrays: every step sets the swarm's coordinates and the per-particle
    viscosity and body force from host arrays, solves with Solver.solve() (PIC
    mapping, DVC weights, assembly, BSSCR solve) and reads the velocity and
    pressure fields back to host numpy arrays."""
    import numpy as np
    import underworld2_gb300 as uw
    dim = cfg["dim"]
    mesh = uw.mesh.FeMesh_Cartesian(elementType="Q1/dQ0", elementRes=cfg["res"], minCoord=(0.0,) * dim,
                                    maxCoord=(1.0,) * dim)
    v = mesh.add_variable(nodeDofCount=dim)
    pr = mesh.subMesh.add_variable(nodeDofCount=1)
    swarm = uw.swarm.Swarm(mesh=mesh)
    visc = swarm.add_variable(dataType="double", count=1)
    force = swarm.add_variable(dataType="double", count=dim)
    swarm.populate_using_layout(uw.swarm.layouts.PerCellRandomLayout(swarm=swarm, particlesPerCell=cfg["ppc"], seed=13))
    axes = "IJK"[:dim]
    walls = [mesh.specialSets["Min%s_VertexSet" % a] + mesh.specialSets["Max%s_VertexSet" % a] for a in axes]
    bc = uw.conditions.DirichletCondition(variable=v, indexSetsPerDof=tuple(walls))
    stokes = uw.systems.Stokes(velocityField=v, pressureField=pr, voronoi_swarm=swarm, conditions=[bc],
                               fn_viscosity=visc, fn_bodyforce=force)
    solver = uw.systems.Solver(stokes)
    solver.set_inner_method("mixed" if mixed else "mg")
    solver.set_inner_rtol(args.inner_rtol)
    solver.set_outer_rtol(1e-8)   # the metric's relative residual
    solver.options.mg.smooth_steps = cfg.get("smooth", 2)
    solver.options.scr.restart = 120
    x_h = np.ascontiguousarray(x_h)
    eta_h = np.ascontiguousarray(eta_h).reshape(-1)
    body_h = np.ascontiguousarray(body_h).reshape(-1, dim)

    def step():
        t0 = time.perf_counter()
        with swarm.deform_swarm():
            swarm.data[:] = x_h
        visc.data[:, 0] = eta_h
        force.data[:] = body_h
        solver.solve()
        vel, p = v.data.copy(), pr.data.copy()
        return time.perf_counter() - t0, vel, p

    for _ in range(min(args.warmup, 1)):
        step()
    ts, out = [], None
    for _ in range(args.steps):
        t, vel, p = step()
        ts.append(t)
        out = (vel, p)
    st = solver.get_stats()
    return {"value": float(np.mean(ts)), "unit": "s/solve",
            "h2d_bytes_per_step": int(x_h.nbytes + eta_h.nbytes + body_h.nbytes),
            "d2h_bytes_per_step": int(out[0].nbytes + out[1].nbytes),
            "api": "uw.systems.Stokes + uw.systems.Solver(...).solve(), swarm coordinates and swarm-variable "
                   "data set from numpy every step, velocity/pressure .data read back",
            "residual": float(st.residual), "pressure_its": int(st.pressure_its)}


def gpu_pairings():
    """GPU solves of the workloads the CPU baseline solves in full (see
    oracle/cpu_reference.pairings): the 2D 64^2 sinker with both Schur
    preconditioners and the 3D GRF workload on 32^3, plain FP64 and mixed."""
    import torch
    from underworld2_gb300._core import Context, rng_seed
    out = {}
    for key, res, pcs in (("sinker2d", (64, 64), ((1, "bfbt"), (0, "uzawa"))), ("grf3d", (32, 32, 32), ((1, "bfbt"),))):
        cfg = dict(CONFIGS[key])
        cfg["res"] = res
        dim = cfg["dim"]
        ctx = Context(dim, res, (0.0,) * dim, (1.0,) * dim)
        ctx.set_bcs(freeslip_mask(ctx))
        x, owner, off, lst, _ = ctx.layout_random(cfg["ppc"], rng_seed(13))
        eta, body = material(cfg, x)
        ip_xi = ctx.pic_map(x, off, lst)
        ip_w = ctx.dvc_weights(off, ip_xi)
        ctx.assemble(off, lst, ip_xi, ip_w, eta, body)
        for pc, name in pcs:
            for mixed in (0, 1):
                best = None
                for _ in range(3):
                    u = ctx.zeros(ctx.n_vdof)
                    p = ctx.zeros(ctx.n_pdof)
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    st = ctx.solve(u, p, mixed=mixed, rtol=1e-8, inner_rtol=1e-10, outer_rtol=1e-9, smooth_steps=2,
                                   restart=120, schur_pc=pc, max_outer=2000)
                    torch.cuda.synchronize()
                    t = time.perf_counter() - t0
                    best = t if best is None else min(best, t)
                out["%s_%s_%s_%s" % (key, "x".join(map(str, res)), name, "mixed" if mixed else "fp64")] = {
                    "solve_s": best, "pressure_its": st["pressure_its"], "velocity_total_its": st["velocity_total_its"],
                    "schur_pc_its": st["schur_pc_its"], "residual": st["residual"]}
        del ctx
    return out


def dram_traffic(kernel_name, config):
    """DRAM bytes (read + write) per launch of the kernel on this workload, from
    the ncu capture recorded in profiles/dram_traffic.json (None if absent)."""
    try:
        d = json.load(open(os.path.join(ROOT, "profiles", "dram_traffic.json")))
        e = d[kernel_name.split(" ")[0] + " " + config]
        return e["dram_bytes_read_per_launch"] + e["dram_bytes_write_per_launch"]
    except Exception:
        return None


def time_kernel_apply(ctx, reps=20):
    """CUDA-event time of the FP32 matrix-free K apply on the finest level.
    Algorithmic bytes per apply: 4*(2*N_v) + 4*M*N_el (x read, y written,
    M equivalent-quadrature weights read: 27 for 3D Q1, 9 for 2D Q1, 25 for
    2D Q2, 125 for 3D Q2)."""
    import torch
    x = torch.randn(ctx.n_vdof, dtype=torch.float32, device=ctx.device)
    y = torch.empty_like(x)
    for _ in range(3):
        ctx._call("uwg_apply_K32", 0, __import__("ctypes").c_void_p(x.data_ptr()), __import__("ctypes").c_void_p(y.data_ptr()))
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(reps):
        ctx._call("uwg_apply_K32", 0, __import__("ctypes").c_void_p(x.data_ptr()), __import__("ctypes").c_void_p(y.data_ptr()))
    e.record()
    torch.cuda.synchronize()
    sec = s.elapsed_time(e) / 1e3 / reps
    nq = (125 if ctx.dim == 3 else 25) if ctx.order == 2 else (27 if ctx.dim == 3 else 9)
    byts = 4 * 2 * ctx.n_vdof + 4 * nq * ctx.n_el
    if ctx.order == 2:
        name = "k_applyK_q2_3d<float>" if ctx.dim == 3 else "k_applyK_q2<float>"
    else:
        name = "k_applyK_q1_3d_tiled<float>" if ctx.dim == 3 else "k_applyK_q1_2d<float>"
    extra = " (+ memset of y)" if (ctx.order == 1 and ctx.dim == 3) else " (+ BC copy)"
    return {"name": name + extra, "seconds": sec, "bytes": byts}


def run_kernel(args):
    """Set the workload up, then launch one operator kernel `--reps` times
    (the target of the ncu captures recorded under profiles/)."""
    import ctypes
    import torch
    from underworld2_gb300._core import Context, rng_seed
    cfg = CONFIGS[args.config]
    dim = cfg["dim"]
    ctx = Context(dim, cfg["res"], (0.0,) * dim, (1.0,) * dim, order=cfg.get("order", 1), porder=cfg.get("porder", 0))
    ctx.set_bcs(freeslip_mask(ctx))
    ppc = args.kernel_ppc or cfg["ppc"]
    x, owner, off, lst, _ = ctx.layout_random(ppc, rng_seed(13))
    eta, body = material(cfg, x)
    ip_xi = ctx.pic_map(x, off, lst)
    ip_w = ctx.dvc_weights(off, ip_xi)
    ctx.assemble(off, lst, ip_xi, ip_w, eta, body)
    torch.cuda.synchronize()
    dt = torch.float32 if args.kernel == "applyK32" else torch.float64
    xv = torch.randn(ctx.n_vdof, dtype=dt, device=ctx.device)
    yv = torch.empty_like(xv)
    name = "uwg_apply_K32" if args.kernel == "applyK32" else "uwg_apply_K64"
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(args.reps):
        ctx._call(name, 0, ctypes.c_void_p(xv.data_ptr()), ctypes.c_void_p(yv.data_ptr()))
    e.record()
    torch.cuda.synchronize()
    print(json.dumps({"kernel": args.kernel, "config": args.config, "reps": args.reps,
                      "ms_per_launch": s.elapsed_time(e) / args.reps}))


def run_gemm(args):
    """The CNN's forward GEMM (BF16 operands, FP32 accumulation, BF16 output)
    on the shape of a 128-channel 3x3 convolution over 16 problems of 128^2
    cells: M = 262144 pixels, N = 128 output channels, K = 9 x 128, `--reps`
    launches on the tcgen05 path and on the mma.sync path."""
    import torch
    from underworld2_gb300._core import Context
    from underworld2_gb300.learned import _Ops
    ops = _Ops(Context(2, (8, 8), (0.0, 0.0), (1.0, 1.0)))
    M, N, K = 262144, 128, 1152
    g = torch.Generator(device="cuda").manual_seed(0)
    A = torch.randn((M, K), device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn((N, K), device="cuda", generator=g).to(torch.bfloat16)
    C = torch.empty((M, N), device="cuda", dtype=torch.bfloat16)
    out = {"kernel": "cnn_gemm", "M": M, "N": N, "K": K, "reps": args.reps}
    for path, name in ((0, "tcgen05"), (1, "mma_sync")):
        ops.set_path(path)
        ops.gemm(M, N, K, A, K, 0, B, K, 1, Cb=C, ldc=N)
        ops.check()
        s_, e_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s_.record()
        for _ in range(args.reps):
            ops.gemm(M, N, K, A, K, 0, B, K, 1, Cb=C, ldc=N)
        e_.record()
        ops.check()
        ms = s_.elapsed_time(e_) / args.reps
        out[name] = {"ms_per_launch": ms, "tflops": 2.0 * M * N * K / ms / 1e9,
                     "hbm_gbs": 2.0 * (M * K + N * K + M * N) / ms / 1e6}
    ops.set_path(0)
    print(json.dumps(out))


def run_rk2(args):
    """`--reps` RK2 steps (FP32 coordinate storage, FP64 arithmetic) through a
    cellular velocity field on the workload's mesh, with --kernel-ppc particles per
    element (the target of the RK2 ncu capture): prints ms per step and particles/s."""
    import torch
    from underworld2_gb300._core import Context, rng_seed
    cfg = CONFIGS[args.config]
    dim = cfg["dim"]
    ctx = Context(dim, cfg["res"], (0.0,) * dim, (1.0,) * dim)
    x, owner, off, lst, _ = ctx.layout_random(args.kernel_ppc or cfg["ppc"], rng_seed(13))
    xyz = torch.stack(torch.meshgrid(*[torch.tensor(a, device=ctx.device) for a in reversed(ctx.axes)],
                                     indexing="ij")[::-1], dim=-1).reshape(-1, dim)
    sn, cs = torch.sin(torch.pi * xyz), torch.cos(torch.pi * xyz)
    vel = torch.zeros_like(xyz)
    vel[:, 0] = sn[:, 0] * cs[:, dim - 1]
    vel[:, dim - 1] = -cs[:, 0] * sn[:, dim - 1]
    vel = vel.contiguous().reshape(-1)
    dt = ctx.max_dt(vel)
    x32 = x.to(torch.float32)
    del x
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctx.rk2(x32, vel, dt)
    torch.cuda.synchronize()
    s.record()
    for _ in range(args.reps):
        ctx.rk2(x32, vel, dt)
    e.record()
    torch.cuda.synchronize()
    ms = s.elapsed_time(e) / args.reps
    print(json.dumps({"kernel": "rk2", "config": args.config, "particles": x32.shape[0], "reps": args.reps,
                      "ms_per_step": ms, "particles_per_s": x32.shape[0] / (ms / 1e3)}))


def run_advdiff(args):
    """SUPG advection-diffusion of T on the workload's Q1 mesh: a cellular
    velocity field, diffusivity 1 at the Gauss points, T fixed on the top and
    bottom walls, `--reps` steps at the Courant time step after 3 untimed.
    Algorithmic bytes per step: the predictor reads phi, phidot, bc (+ writes
    phi, phidot); each of the two corrector passes reads phi, phidot, the
    velocity and the 3^d Gauss-point diffusivities and writes R (+ M once),
    then reads R, M, bc, phi, phidot and writes phi, phidot."""
    import torch
    from underworld2_gb300._core import Context
    cfg = CONFIGS[args.config]
    dim = cfg["dim"]
    ctx = Context(dim, cfg["res"], (0.0,) * dim, (1.0,) * dim)
    xyz = torch.stack(torch.meshgrid(*[torch.tensor(a, device=ctx.device) for a in reversed(ctx.axes)],
                                     indexing="ij")[::-1], dim=-1).reshape(-1, dim)
    s, c = torch.sin(torch.pi * xyz), torch.cos(torch.pi * xyz)
    vel = torch.zeros_like(xyz)
    vel[:, 0] = s[:, 0] * c[:, dim - 1]
    vel[:, dim - 1] = -c[:, 0] * s[:, dim - 1]
    vel = (1e3 * vel).contiguous().reshape(-1)
    nq = 3 ** dim
    kappa = torch.ones(ctx.n_el * nq, dtype=torch.float64, device=ctx.device)
    top, bot = xyz[:, dim - 1] == 1.0, xyz[:, dim - 1] == 0.0
    bc = (top | bot).to(torch.uint8)
    phi = (1.0 - xyz[:, dim - 1]).contiguous()
    phidot = torch.zeros_like(phi)
    bcval = phi.clone()
    dt = ctx.advdiff_max_dt(vel, kappa)
    for _ in range(3):
        ctx.advdiff_step(dt, vel, kappa, phi, phidot, bc, bcval)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.reps):
        ctx.advdiff_step(dt, vel, kappa, phi, phidot, bc, bcval)
    ev1.record()
    torch.cuda.synchronize()
    sec = ev0.elapsed_time(ev1) / 1e3 / args.reps
    n, ne = ctx.n_nodes, ctx.n_el
    byts = (8 * 4 * n + n) + 2 * (8 * (2 + dim) * n + 8 * nq * ne + 8 * n) + 8 * n + 2 * (8 * 6 * n + n)
    print(json.dumps({"kernel": "advdiff", "config": args.config, "res": list(ctx.res), "reps": args.reps, "dt": dt,
                      "ms_per_step": sec * 1e3, "algorithmic_bytes_per_step": byts,
                      "GBps": byts / sec / 1e9, "T_finite": bool(torch.isfinite(phi).all()),
                      "T_range": [float(phi.min()), float(phi.max())]}))


def run_slcn(args):
    """SLCN advection-diffusion of T on the workload's Q1 mesh (same cellular
    velocity, diffusivity 1e-3 at the 5^d Gauss points, T fixed on the top and
    bottom walls): `--reps` steps of departure values + Crank-Nicolson CG solve
    (relative residual 1e-10) at dt = min(dx / v_max, dx^2 / kappa) after 3
    untimed steps.  Reported with the CG iteration count of the last step."""
    import torch
    from underworld2_gb300._core import Context
    cfg = CONFIGS[args.config]
    dim = cfg["dim"]
    ctx = Context(dim, cfg["res"], (0.0,) * dim, (1.0,) * dim)
    xyz = torch.stack(torch.meshgrid(*[torch.tensor(a, device=ctx.device) for a in reversed(ctx.axes)],
                                     indexing="ij")[::-1], dim=-1).reshape(-1, dim)
    s, c = torch.sin(torch.pi * xyz), torch.cos(torch.pi * xyz)
    vel = torch.zeros_like(xyz)
    vel[:, 0] = s[:, 0] * c[:, dim - 1]
    vel[:, dim - 1] = -c[:, 0] * s[:, dim - 1]
    vmax = float(vel.norm(dim=1).max()) * 1e3
    vel = (1e3 * vel).contiguous().reshape(-1)
    kappa = torch.full((ctx.n_el * 5 ** dim,), 1e-3, dtype=torch.float64, device=ctx.device)
    bc = ((xyz[:, dim - 1] == 1.0) | (xyz[:, dim - 1] == 0.0)).to(torch.uint8)
    phi = (1.0 - xyz[:, dim - 1]).contiguous()
    dt = min(ctx.min_sep / vmax, ctx.min_sep ** 2 / 1e-3)
    st = {}

    def step():
        ps = ctx.slcn_phistar(dt, vel, phi)
        st["its"], st["res"] = ctx.slcn_solve(dt, kappa, bc, ps, phi, rtol=1e-10)

    for _ in range(3):
        step()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.reps):
        step()
    ev1.record()
    torch.cuda.synchronize()
    sec = ev0.elapsed_time(ev1) / 1e3 / args.reps
    print(json.dumps({"kernel": "slcn", "config": args.config, "res": list(ctx.res), "reps": args.reps, "dt": dt,
                      "ms_per_step": sec * 1e3, "cg_iterations": st["its"], "cg_residual": st["res"],
                      "T_finite": bool(torch.isfinite(phi).all()),
                      "T_range": [float(phi.min()), float(phi.max())]}))


def run_learned(args):
    """Learned warm start and coarse-level correction on the 2D 128^2 Q1/dQ0
    problem family of the training set (log10 viscosity GRF with correlation
    length U[0.05, 0.2] and contrast 10^U[3,6], 0-8 inclusions of radius
    U[0.03, 0.1] with density +-1, 20 particles per element, free slip):
    generate `--train` solves with the plain path and train the CNN (skipped
    with --train 0), then on `--eval` held-out seeds compare outer (Schur
    FGMRES) iterations and time to a 1e-8 residual of
      fp64            the plain FP64 solve,
      mixed           the mixed-precision solve from zero,
      mixed_coarse    the same with the coarse-level correction (aggregates of
                      --coarse-agg cells; its setup on a fresh assembly is timed),
      learned         mixed, the network's pressure as the first search direction,
      guess           mixed, the network's pressure as the initial guess,
      learned_coarse  learned + the coarse-level correction,
      hydro           mixed, the hydrostatic pressure (an input channel) as the
                      first direction (control),
    prediction time included in the learned arms.  Problems without buoyancy
    (no inclusions: zero solution) are left out of the statistics."""
    import numpy as np
    import torch
    from underworld2_gb300 import learned
    ps = learned.ProblemSet(res=128, ppc=20)
    net, t_gen, t_train, losses = None, 0.0, 0.0, []
    if args.train > 0:
        t0 = time.perf_counter()
        X, Y = learned.generate(ps, list(range(1000, 1000 + args.train)))
        torch.cuda.synchronize()
        t_gen = time.perf_counter() - t0
        net = learned.WarmStartNet(ps.ctx, seed=0)
        t0 = time.perf_counter()
        losses = learned.train(net, X, Y, epochs=args.epochs, batch=8)
        torch.cuda.synchronize()
        t_train = time.perf_counter() - t0
        del X, Y
    agg_c = args.coarse_agg
    rows = []
    ev = lambda: torch.cuda.Event(enable_timing=True)
    for s in range(900000, 900000 + args.eval):
        f, scales = ps.assemble(s)
        r = {}
        u64, p64, st = ps.solve(0)
        r.update(fp64_its=st["pressure_its"], fp64_s=st["total_time"], res=st["residual"])
        _, _, st = ps.solve(1)
        r.update(mixed_its=st["pressure_its"], mixed_s=st["total_time"], res=max(r["res"], st["residual"]))
        ps.assemble(s)   # fresh assembly: the coarse operator is built (and timed) inside the solve
        _, _, st = ps.solve(1, coarse_agg=agg_c)
        r.update(mixed_coarse_its=st["pressure_its"], mixed_coarse_s=st["total_time"],
                 coarse_setup_s=st["coarse_setup_time"], res=max(r["res"], st["residual"]))
        pt = p64 - p64.mean()
        nt = max(float(pt.norm()), 1e-300)
        r["trivial"] = float(pt.norm()) == 0.0
        if net is not None:
            e0, e1 = ev(), ev()
            e0.record()
            p0 = learned.predict_pressure(net, f, scales)
            e1.record()
            torch.cuda.synchronize()
            t_pred = e0.elapsed_time(e1) / 1e3
            _, _, stl, fb = learned.solve_with_warm_start(ps, net, f, scales, mode="direction")
            _, _, stg, fbg = learned.solve_with_warm_start(ps, net, f, scales, mode="guess")
            ps.assemble(s)
            _, _, stc, fbc = learned.solve_with_warm_start(ps, net, f, scales, mode="direction", coarse_agg=agg_c)
            ph = (f[:, :, 2].reshape(-1).double() * scales[1]).contiguous()
            _, _, sth = ps.solve(1, p_dir=ph)
            r.update(learned_its=stl["pressure_its"], learned_s=stl["total_time"] + t_pred,
                     guess_its=stg["pressure_its"], guess_s=stg["total_time"] + t_pred,
                     learned_coarse_its=stc["pressure_its"], learned_coarse_s=stc["total_time"] + t_pred,
                     hydro_its=sth["pressure_its"], hydro_s=sth["total_time"], predict_s=t_pred,
                     fallback=bool(fb or fbg or fbc), p_rel_err=float((p0 - pt).norm() / nt),
                     hydro_p_rel_err=float((ph - ph.mean() - pt).norm() / nt),
                     res=max(r["res"], stl["residual"], stg["residual"], stc["residual"], sth["residual"]))
        rows.append(r)
    nt_rows = [r for r in rows if not r["trivial"]]
    arms = ["fp64", "mixed", "mixed_coarse"] + (["learned", "guess", "learned_coarse", "hydro"] if net else [])
    stat = lambda k, f_: float(f_([r[k] for r in nt_rows]))
    out = {
        "workload": "2D 128^2 Q1/dQ0 learned-set problems, 20 particles per cell, free slip, rtol 1e-8",
        "train_solves": args.train, "eval_solves": args.eval, "nontrivial": len(nt_rows), "epochs": args.epochs,
        "coarse_agg": agg_c, "generate_s": t_gen, "train_s": t_train,
        "loss_first_epoch": losses[0] if losses else None, "loss_last_epoch": losses[-1] if losses else None,
        "params": net.n_params() if net else 0,
        "its_mean": {a: stat(a + "_its", np.mean) for a in arms},
        "s_mean": {a: stat(a + "_s", np.mean) for a in arms},
        "s_median": {a: stat(a + "_s", np.median) for a in arms},
        "coarse_setup_s_median": stat("coarse_setup_s", np.median),
        "max_residual": float(max(r["res"] for r in rows)),
        "faster_than_mixed": {a: int(sum(r[a + "_s"] < r["mixed_s"] for r in nt_rows)) for a in arms},
    }
    if net is not None:
        out.update(p_rel_err_mean=stat("p_rel_err", np.mean), p_rel_err_median=stat("p_rel_err", np.median),
                   hydro_p_rel_err_mean=stat("hydro_p_rel_err", np.mean), predict_s_mean=stat("predict_s", np.mean),
                   fallbacks=int(sum(r["fallback"] for r in nt_rows)))
    print(json.dumps(out))


def run_convection(args):
    """Thermal-convection time loop of the 3D Q2/dPc1 configuration
    (`--config conv3d_q2` or `conv3d_q2_small`), `--steps` steps after one
    untimed: T lives on the Q1 mesh of the same elements (T = 1 at the bottom,
    0 at the top, initial 1 - z + seeded 1e-2 noise, diffusivity 1); per step
    T is sampled at the particles, viscosity exp(-9.2 T) and buoyancy Ra T
    (Ra = 1e6) are assembled, the Stokes system is solved in mixed precision
    from the previous pressure, T is advanced by one SUPG step with the
    velocity at the Q1 nodes, and the particles by one RK2 step, all at the
    smaller of the particle and SUPG Courant steps.  A mixed solve that does
    not converge falls back to the plain FP64 path.  Every tenth step the plain
    FP64 solve of the same system is run beside the mixed one (time, residual
    and the relative difference of the two velocity fields).  The warm start is
    the previous step's pressure; there is no 3D network."""
    import numpy as np
    import torch
    from underworld2_gb300._core import Context, rng_seed
    cfg = CONFIGS[args.config]
    assert cfg.get("order", 1) == 2 and cfg["dim"] == 3, "convection loop: a 3D Q2/dPc1 config"
    res = cfg["res"]
    ctx = Context(3, res, (0.0,) * 3, (1.0,) * 3, order=2, porder=1)
    ctx.set_bcs(freeslip_mask(ctx))
    tctx = Context(3, res, (0.0,) * 3, (1.0,) * 3)
    x, owner, off, lst, _ = ctx.layout_random(cfg["ppc"], rng_seed(13))
    nq = [r + 1 for r in res]
    zz, yy, xx = torch.meshgrid(*[torch.tensor(a, device=ctx.device) for a in reversed(tctx.axes)], indexing="ij")
    g = torch.Generator(device="cpu").manual_seed(7)
    a = (torch.rand(4, 3, generator=g, dtype=torch.float64) * 2.0 - 1.0).tolist()
    noise = sum(a[k - 1][0] * torch.cos(torch.pi * k * xx + a[k - 1][1]) * torch.cos(torch.pi * k * yy + a[k - 1][2])
                for k in range(1, 5)) * torch.sin(torch.pi * zz) / 4.0
    T = (1.0 - zz + 0.01 * noise).clamp(0.0, 1.0).reshape(-1).contiguous()
    Tdot = torch.zeros_like(T)
    tbc = ((zz == 0.0) | (zz == 1.0)).reshape(-1).to(torch.uint8)
    Tbc = T.clone()
    kappa = torch.ones(tctx.n_el * 27, dtype=torch.float64, device=ctx.device)
    u = ctx.zeros(ctx.n_vdof)
    p = ctx.zeros(ctx.n_pdof)
    n2 = [2 * r + 1 for r in res]
    opts = dict(rtol=1e-8, inner_rtol=1e-10, outer_rtol=1e-9, smooth_steps=2, restart=120, schur_pc=0, max_outer=500)
    ev = lambda: torch.cuda.Event(enable_timing=True)
    rec = []

    from underworld2_gb300._native import UwgError
    fallbacks = [0]
    compare = []

    def step(timed, k=0):
        e = [ev() for _ in range(6)]
        e[0].record()
        Tp = tctx.interpolate_field(x, T, 1)[0][:, 0]
        eta = torch.exp(-9.2 * Tp).contiguous()
        body = torch.zeros_like(x)
        body[:, 2] = 1e6 * Tp
        ip_xi = ctx.pic_map(x, off, lst)
        n_in = int(off[-1])
        diag = {"nan_positions": int(torch.isnan(x).any(dim=1).sum()), "listed": n_in,
                "max_abs_xi": float(ip_xi[:n_in].abs().max()) if n_in else 0.0,
                "max_per_cell": int((off[1:] - off[:-1]).max())}
        if diag["nan_positions"] or diag["max_abs_xi"] > 1.0 + 1e-9:
            raise RuntimeError("convection loop: inconsistent particle state %s" % diag)
        ip_w = ctx.dvc_weights(off, ip_xi)
        ctx.assemble(off, lst, ip_xi, ip_w, eta, body.contiguous())
        e[5].record()
        if timed and k % 10 == 0:
            # the plain FP64 path on this step's system, from the same start
            u64, p64 = u.clone(), p.clone()
            t0 = time.perf_counter()
            st64 = ctx.solve(u64, p64, mixed=0, zero_guess=0, **opts)
            torch.cuda.synchronize()
            t64 = time.perf_counter() - t0
        u_start, p_start = u.clone(), p.clone()
        e[1].record()
        try:
            st = ctx.solve(u, p, mixed=1, zero_guess=0, **opts)
        except UwgError:
            fallbacks[0] += 1
            u.copy_(u_start)
            p.copy_(p_start)
            st = ctx.solve(u, p, mixed=0, zero_guess=0, **opts)
        del u_start, p_start
        if not bool(torch.isfinite(u).all()):
            raise RuntimeError("convection loop: non-finite velocity %s" % st)
        e[2].record()
        uq1 = u.reshape(n2[2], n2[1], n2[0], 3)[::2, ::2, ::2].contiguous().reshape(-1)
        dt = min(ctx.max_dt(u), tctx.advdiff_max_dt(uq1, kappa))
        tctx.advdiff_step(dt, uq1, kappa, T, Tdot, tbc, Tbc)
        e[3].record()
        ctx.rk2(x, u, dt)
        lost = ctx.update_owners(x, owner, off, lst)
        e[4].record()
        diag["lost"] = lost
        diag["dt"] = dt
        torch.cuda.synchronize()
        if timed and k % 10 == 0:
            compare.append({"step": k, "fp64_solve_s": t64, "fp64_outer_its": st64["pressure_its"],
                            "fp64_residual": st64["residual"], "mixed_outer_its": st["pressure_its"],
                            "mixed_residual": st["residual"],
                            "velocity_rel_diff": float(torch.linalg.norm(u - u64) / torch.linalg.norm(u64))})
            del u64, p64
        if timed:
            ph = [e[0].elapsed_time(e[5]) / 1e3, e[1].elapsed_time(e[2]) / 1e3, e[2].elapsed_time(e[3]) / 1e3,
                  e[3].elapsed_time(e[4]) / 1e3]
            rec.append({"assemble_s": ph[0], "solve_s": ph[1], "advdiff_s": ph[2], "advect_s": ph[3],
                        "step_s": sum(ph), "dt": dt, "outer_its": st["pressure_its"],
                        "residual": st["residual"], "T_mean": float(T.mean()), "vrms_proxy": float(u.norm()),
                        "particles": diag})

    step(False)
    for k in range(args.steps):
        step(True, k)
    agg = lambda k: float(np.mean([r[k] for r in rec]))
    print(json.dumps({"convection": workload_name(args.config), "steps": args.steps,
                      "per_step_s": agg("step_s"), "phases_s": {k: agg(k) for k in ("assemble_s", "solve_s",
                                                                                     "advdiff_s", "advect_s")},
                      "mean_outer_its": agg("outer_its"), "max_residual": max(r["residual"] for r in rec),
                      "fallbacks_to_fp64": fallbacks[0], "learned": "none (no 3D network)",
                      "vs_plain_fp64": compare,
                      "per_step": [[round(r["step_s"], 4), r["outer_its"], r["residual"]] for r in rec],
                      "particles_last": rec[-1]["particles"], "T_mean_last": rec[-1]["T_mean"]}))


def run_profile_solve(args):
    """One map + DVC + assembly + solve of the workload, untimed (the target of
    the launch-list captures recorded under profiles/); `--kernel-ppc` lowers
    the particle count to keep the device footprint small."""
    import torch
    from underworld2_gb300._core import Context, rng_seed
    cfg = CONFIGS[args.config]
    dim = cfg["dim"]
    ctx = Context(dim, cfg["res"], (0.0,) * dim, (1.0,) * dim, order=cfg.get("order", 1), porder=cfg.get("porder", 0))
    ctx.set_bcs(freeslip_mask(ctx))
    ppc = args.kernel_ppc or cfg["ppc"]
    x, owner, off, lst, _ = ctx.layout_random(ppc, rng_seed(13))
    eta, body = material(cfg, x)
    ip_xi = ctx.pic_map(x, off, lst)
    ip_w = ctx.dvc_weights(off, ip_xi)
    ctx.assemble(off, lst, ip_xi, ip_w, eta, body)
    u, p = ctx.zeros(ctx.n_vdof), ctx.zeros(ctx.n_pdof)
    st = ctx.solve(u, p, mixed=1 if args.mode == "mixed" else 0, rtol=1e-8, inner_rtol=args.inner_rtol,
                   outer_rtol=args.outer_rtol, smooth_steps=cfg.get("smooth", 2), restart=120, schur_pc=args.schur_pc if cfg.get("porder", 0) == 0 else 0,
                   schur_pc_rtol=args.bfbt_rtol, schur_pc_its=args.bfbt_its, max_outer=args.max_outer)
    torch.cuda.synchronize()
    print(json.dumps({"profile_solve": args.config, "particles_per_cell": ppc,
                      "pressure_its": st["pressure_its"], "schur_pc_its": st["schur_pc_its"],
                      "velocity_total_its": st["velocity_total_its"], "residual": st["residual"],
                      "total_time": st["total_time"]}))


def count_launches(ctx, x0, owner0, off0, lst0, eta0, body0, mixed, opts, u, p):
    """Kernels launched by libuwg in one solve step and in one advection step,
    counted with the CUDA activity profiler."""
    import torch
    from torch.profiler import ProfilerActivity, profile
    x, owner, off, lst = x0.clone(), owner0.clone(), off0.clone(), lst0.clone()
    # libuwg's kernels are named k_* / vk_*, some inside an anonymous namespace
    # ("void (anonymous namespace)::k_applyK_q2_3d<...>(...)")
    ours = re.compile(r"(^|[\s:])v?k_\w")

    def count(prof):
        n = 0
        for evt in prof.events():
            name = evt.name or ""
            if evt.device_type.name == "CUDA" and (ours.search(name.split("(")[0] if "::" not in name else name)
                                                    or "uwg" in name):
                n += 1
        return n

    with profile(activities=[ProfilerActivity.CUDA]) as prof:
        ip_xi = ctx.pic_map(x, off, lst)
        ip_w = ctx.dvc_weights(off, ip_xi)
        ctx.assemble(off, lst, ip_xi, ip_w, eta0, body0)
        u.zero_(); p.zero_()
        ctx.solve(u, p, mixed=mixed, **opts)
        torch.cuda.synchronize()
    n_solve = count(prof)
    x32 = x0.to(torch.float32)
    with profile(activities=[ProfilerActivity.CUDA]) as prof:
        dt = ctx.max_dt(u)
        ctx.rk2(x32, u, dt)
        ctx.update_owners(x32, owner, off, lst)
        torch.cuda.synchronize()
    return n_solve, count(prof)


# ---------------------------------------------------------------------------
# CPU arm: the oracle (reference algorithms restated in C) on host cores
# ---------------------------------------------------------------------------
def cpu_baseline(args):
    """The CPU port on this workload, one bounded sample (the `cpu_baseline` of our line)."""
    from oracle import cpu_reference
    try:
        return cpu_reference.measure(CONFIGS[args.config], workload_name(args.config), steps=1)
    except NotImplementedError as e:
        return {"unavailable": str(e)}


def run_reference(args):
    """The reference arm: the CPU port of the path on all host cores (the reference
    itself cannot be built here), set up once at full size, then `--warmup` +
    `--steps` bounded samples; plus full CPU solves of the paired workloads."""
    from oracle import cpu_reference
    try:
        b = cpu_reference.CPUBaseline(CONFIGS[args.config], workload_name(args.config))
    except NotImplementedError as e:
        return {"impl": "reference", "unavailable": str(e)}
    for _ in range(args.warmup):
        b.step()
    t0 = time.perf_counter()
    samples = [b.step() for _ in range(args.steps)]
    wall = time.perf_counter() - t0
    res = b.result(samples)
    res["pairings"] = cpu_reference.pairings(CONFIGS)
    line = {
        "impl": "reference",
        "metric": "Stokes solve time @1e-8 resid (learned+FP32 vs FP64 GPU); particles/s advected",
        "value": res["value"],
        "unit": "s/solve",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "ms_per_step": 1e3 * wall / max(args.steps, 1),
        "config": workload_config(args.config),
        "particles_per_s": res.get("particles_per_s"),
        "cpu_baseline": res,
        "e2e": {"value": res["value"], "unit": "s/solve", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="grf3d", choices=sorted(CONFIGS))
    ap.add_argument("--mode", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--inner-rtol", type=float, default=1e-10)
    ap.add_argument("--outer-rtol", type=float, default=1e-9)
    ap.add_argument("--schur-pc", type=int, default=1, help="0: Uzawa S^ (reference), 1: scaled BFBt")
    ap.add_argument("--bfbt-rtol", type=float, default=3e-2)
    ap.add_argument("--bfbt-its", type=int, default=0, help="> 0: fixed CG iterations per BFBt L-solve")
    ap.add_argument("--kernel", choices=["applyK32", "applyK64", "advdiff", "slcn", "rk2", "cnn_gemm"],
                    help="only launch one operator kernel, or time SUPG / SLCN advection-diffusion steps (profiling)")
    ap.add_argument("--kernel-ppc", type=int, default=0)
    ap.add_argument("--profile-solve", action="store_true", help="one untimed solve (profiling target)")
    ap.add_argument("--convection", action="store_true",
                    help="time the 3D Q2/dPc1 thermal-convection loop (advection-diffusion + Stokes + RK2)")
    ap.add_argument("--learned", action="store_true",
                    help="train the warm-start CNN on generated 2D 128^2 solves and evaluate it on held-out seeds")
    ap.add_argument("--train", type=int, default=800)
    ap.add_argument("--eval", type=int, default=100)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--coarse-agg", type=int, default=8, help="aggregate size of the coarse-level correction")
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--max-outer", type=int, default=500)
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-count-launches", dest="count_launches", action="store_false")
    args = ap.parse_args()
    if args.kernel == "advdiff":
        run_advdiff(args)
        return
    if args.kernel == "rk2":
        run_rk2(args)
        return
    if args.kernel == "slcn":
        run_slcn(args)
        return
    if args.kernel == "cnn_gemm":
        run_gemm(args)
        return
    if args.kernel:
        run_kernel(args)
        return
    if args.profile_solve:
        run_profile_solve(args)
        return
    if args.learned:
        run_learned(args)
        return
    if args.convection:
        run_convection(args)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference(args)))
        return
    if world > 1:
        # replicas only: every rank runs the same single-GPU workload on its own device
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
        dist.barrier()
        line = combine_replicas(run_gpu(args), world, "cuda")
        if rank == 0:
            print(json.dumps(line))
        dist.destroy_process_group()
        return
    print(json.dumps(run_gpu(args)))


def combine_replicas(line, world, device):
    """Replicas only: every rank solved its own copy of the workload.  Times are
    the maximum over ranks (the job ends with the slowest replica), throughputs
    the whole job's (all ranks' particles over that time)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([line["value"], line["ms_per_step"], line["e2e"]["value"],
                      line["particles_per_s"] ** -1 if line.get("particles_per_s") else 0.0],
                     dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    line["value"], line["ms_per_step"], line["e2e"]["value"] = float(t[0]), float(t[1]), float(t[2])
    if line.get("particles_per_s"):
        line["particles_per_s"] = world / float(t[3])
    line["n_gpus"] = world
    line["config"]["parallelism"] = "replicas x%d" % world
    return line


if __name__ == "__main__":
    main()
