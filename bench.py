#!/usr/bin/env python3
"""Benchmark of the GB300 eMix3d hot path: Mcell-RK3-steps/s.

One step = one full RK3 step (three substeps: compact velocity gradients,
SGS viscosity, fluxes, compact flux divergence, RK update, WENO5 level-set
stage) of the 256^3 wall-bounded stirred-tank workload (Lele-6 compact
scheme with 3rd/4th-order closures, Smagorinsky Cs = 0.1, CFL 0.3), FP64.
Fields are seeded synthetic data of that configuration.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun every rank advances its own independent replica of the grid
(the path has no exchange step), so ``value`` is the sum over ranks and the
scaling is weak.  ``--impl reference`` times the CPU restatement of the
reference's algorithm (the oracle) on all host threads, rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_GRID = 256
SINGLE_N = 128           # grid of the single-thread CPU sample (same generator)
G = 5                    # level-set ghost layers


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


# Cells one launch of each kernel class covers, averaged over its launches in
# a step.  The level-set stages cover the padded grid (stage 1), the grid
# grown by the 3-cell WENO5 reach (stage 2) and the interior (stage 3).
def cells_per_launch(name: str, dims, g: int) -> float:
    nx, ny, nz = dims
    n = nx * ny * nz
    if name == "weno_stage":
        return ((nx + 2 * g) * (ny + 2 * g) * (nz + 2 * g) + (nx + 6) * (ny + 6) * (nz + 6) + n) / 3.0
    if name == "ghost_pad":
        return (nx + 2 * g) * (ny + 2 * g) * (nz + 2 * g)
    return n


# Algorithmic bytes per launch of each kernel class, per cell of the grid
# (n = cells, ng = ghost-padded cells of the level-set grid): every field a
# kernel must read or write, once.
def algorithmic_bytes(name: str, n: int, ng: int, sgs: int = 1, dims=None, g: int = 5) -> float:
    d = 8.0
    if name == "weno_stage":
        # per stage: phi_s over the stage's region, phi_0 (stages 2, 3), u (3n)
        # and jbn (3n) read once, phi_out over the region written
        nx, ny, nz = dims
        r = ((nx + 2 * g) * (ny + 2 * g) * (nz + 2 * g), (nx + 6) * (ny + 6) * (nz + 6), n)
        return d * (2 * r[0] + 6 * n + 3 * r[1] + 6 * n + 3 * r[2] + 6 * n) / 3.0
    if name in ("grad_x", "grad_y", "grad_z"):
        return d * 6 * n           # 3 in, 3 out
    if name == "grad_yz":
        return d * 9 * n           # 3 in (read once), 6 out
    if name == "div_x":
        return d * 10 * n          # 5 in, 5 out
    if name in ("div_y", "div_z"):
        return d * 15 * n          # 5 in, 5 accumulated (read + write)
    if name == "flux":
        return d * 40 * n          # um 5, u 3, p, dvel 9, vis, jbn 3, J*metric 3 -> 15
    if name == "sgs_flux":
        return d * 41 * n          # the flux reads with dxyz for vis -> vis and the 15 fluxes
    if name == "sgs":
        return d * (14 if sgs == 1 else 20) * n
    if name == "rk_post":
        return d * (17 * 2 + 12) / 3.0 * n + d * 9 * n
    if name == "prim":
        return d * 8 * n
    if name == "ghost_pad":
        return d * (n + ng)
    return 0.0


# wall boundary conditions of the tank (frontera_z/y/x_val) in every substep
WALLS = 1
# the impeller as a rotating volumetric forcing (rushton(sub_step)) in every substep
IMPELLER = True

# FP64 operations (dfma + dadd + dmul thread instructions) per cell a launch
# covers, measured with ncu on the 192^3 tank (profiles/step_kernels_full_
# stirred_tank_192.txt, profiles/weno_stage_stirred_tank_192.txt).
FP64_OPS_PER_CELL = {
    "weno_stage": 115.4, "grad_x": 18.0, "grad_y": 18.0, "grad_z": 18.0, "grad_yz": 36.1,
    "div_x": 30.1, "div_y": 30.2, "div_z": 30.2, "flux": 43.0, "sgs": 28.0, "sgs_flux": 58.0,
    # the RK update: 19.9 in substep 1, 29.5 in substeps 2 and 3 (their um term)
    "rk_post": 26.3,
}

# DRAM bytes (read + write) per cell a launch covers, from the same ncu
# captures; the bench scales them to the 256^3 launch by its cells.
DRAM_BYTES_PER_CELL = {"weno_stage": 89.1}

# where the two tables above come from: ncu captures of the named commands,
# summarised (command, counters, per-kernel figures) in the profiles files
CONSTANT_SOURCES = {
    "fp64_ops_per_cell": "ncu --set full (FP64 fma + add + mul thread instructions per cell), "
                         "python -m emix_gb300.run --n 192 --steps 2 --walls --impeller: "
                         "profiles/step_kernels_full_stirred_tank_192.txt, "
                         "profiles/weno_stage_stirred_tank_192.txt",
    "dram_bytes_per_cell": "ncu --set full (dram__bytes_read.sum + dram__bytes_write.sum per cell of the "
                           "stage region), same capture: profiles/weno_stage_stirred_tank_192.txt",
}


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-f", self.path], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.proc is None:
            return out
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        try:
            for line in Path(self.path).read_text().splitlines():
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        finally:
            try:
                os.unlink(self.path)
            except OSError:
                pass
        if not rows:
            return out
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        out.update(sm_mhz=float(np.median(sm)) if sm else None,
                   sm_max_mhz=max(mx) if mx else None, reasons=reasons, samples=len(rows))
        return out


def dist_setup():
    from emix_gb300 import replicas
    return replicas.world_from_env()


def cpu_sample(n: int, steps: int, warmup: int, threads: int = 0, w=None):
    """Oracle (CPU restatement of the reference algorithm) stepping the n^3
    tank (the headline generator and settings) on `threads` host threads (0:
    all).  Returns (Mcell-steps/s, seconds, threads)."""
    from emix_gb300 import fields as F
    from oracle import oracle_py as O
    O.load()
    before = O.get_threads()
    if threads:
        O.set_threads(threads)
    try:
        w = w if w is not None else F.stirred_tank(n=n, impeller=IMPELLER)
        p = O.step_params(w, bc_walls=WALLS)
        d, r = O.inisgdm(np.ascontiguousarray(w.grid.coords()))
        um, phi = w.um, w.phi
        for _ in range(warmup):
            um, phi = O.step(p, um, phi, w.jbn, w.mask, d, r)
        t0 = time.perf_counter()
        for _ in range(steps):
            um, phi = O.step(p, um, phi, w.jbn, w.mask, d, r)
        sec = time.perf_counter() - t0
        thr = O.get_threads()
    finally:
        O.set_threads(before)
    return w.grid.ncell * steps / sec / 1e6, sec, thr


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    # the headline workload itself (256^3 tank), every step a full RK3 step of
    # it; the CPU needs no warm-up beyond its first step
    warm = min(args.warmup, 1)
    v, sec, thr = cpu_sample(N_GRID, args.steps, warm)
    line = {
        "impl": "reference", "metric": "Mcell-RK3-steps/s", "value": round(v, 4),
        "unit": "Mcell-RK3-steps/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": warm, "ms_per_step": round(1e3 * sec / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": config_dict(None),
        "cpu_baseline": {"value": round(v, 4), "unit": "Mcell-RK3-steps/s", "cores": thr,
                         "kind": "port",
                         "sample": f"{args.steps} RK3 steps of the {N_GRID}^3 stirred tank (the "
                                   f"workload of the config, {warm} untimed step first), CPU "
                                   f"restatement of the reference algorithm, {thr} threads"},
        "e2e": {"value": round(v, 4), "unit": "Mcell-RK3-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def ensemble_leg(steps: int, warmup: int, stream=None, world: int = 1, rank: int = 0):
    """The uneven 48-grid ensemble (seed 7): batched persistent launches (autotuned,
    graph-replayed) against the same grids stepped one by one (each grid's own
    graph).  Under torchrun the grids are split between the ranks (largest
    first, to the least-loaded rank; no collective on the data path) and the
    job's time is the slowest rank's.  Returns a dict for the JSON line."""
    import torch
    from emix_gb300 import fields as F
    from emix_gb300 import ops
    from emix_gb300 import replicas
    costs = [nx * ny * nz for nx, ny, nz in F.ensemble_shapes(48, 7)]
    total_cells = sum(costs)
    part = replicas.shard_by_cost(costs, world)[rank]
    ws = F.ensemble(ngrids=48, seed=7, only=set(part))
    b = ops.Batch(ws)
    s = stream or torch.cuda.Stream()
    b.set_stream(s.cuda_stream)
    tuned_ms = b.autotune(nsteps=2)
    ncell = b.ncell

    def timed(fn):
        b.upload()
        fn(warmup)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(s)
        fn(steps)
        e1.record(s)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    replicas.barrier(world)
    ms_b = replicas.max_over_ranks(timed(lambda k: b.step(k, use_graph=True)), world)
    replicas.barrier(world)
    ms_g = replicas.max_over_ranks(timed(lambda k: b.step_per_grid(k, use_graph=True)), world)
    replicas.barrier(world)
    ms_e = replicas.max_over_ranks(timed(lambda k: b.step_per_grid(k, use_graph=False)), world)
    # the batched result agrees with the per-grid result (to rounding)
    b.upload(); b.step(1, use_graph=True); a0 = b.download(0)[0]
    b.upload(); b.step_per_grid(1, use_graph=True); a1 = b.download(0)[0]
    diff = replicas.max_over_ranks(float(np.max(np.abs(a0 - a1)) / np.max(np.abs(a1))), world)
    tune = b.tuning()
    b.close()
    return {
        "workload": "48 periodic grids, nx,ny,nz each from {32,48,...,160} (seed 7), omega~U[0.5,2]",
        "cells": total_cells, "steps": steps, "ranks": world,
        "grids_per_rank": len(part), "cells_rank0": ncell,
        "batched": {"value": round(total_cells / (ms_b * 1e-3) / 1e6, 3), "ms_per_step": round(ms_b, 3)},
        "per_grid": {"value": round(total_cells / (ms_g * 1e-3) / 1e6, 3), "ms_per_step": round(ms_g, 3),
                     "form": "each grid's own captured graph, grids one after another"},
        "per_grid_eager": {"value": round(total_cells / (ms_e * 1e-3) / 1e6, 3), "ms_per_step": round(ms_e, 3),
                           "form": "each grid's plain kernels launched one by one, no graph"},
        "speedup": round(ms_g / ms_b, 3), "speedup_vs_eager": round(ms_e / ms_b, 3),
        "max_rel_diff_vs_per_grid": diff,
        "tuning": {"cells_per_thread": tune[0], "yz_block": tune[1], "ctas_per_sm": tune[2],
                   "autotune_best_ms": round(tuned_ms, 3)},
    }


def large_leg(steps: int, warmup: int, stream=None):
    """The 512 x 512 x 384 tank (same generator and settings as the headline
    workload): device-resident graph-replayed steps and the context's device
    footprint.  Returns a dict for the JSON line."""
    import torch
    from emix_gb300 import fields as F
    from emix_gb300 import ops
    w = F.stirred_tank(n=512, nz=384, impeller=IMPELLER)
    ctx = ops.Context(w, level_set=True, ls_ghost=G, bc_walls=WALLS)
    s = stream or torch.cuda.Stream()
    ctx.set_stream(s.cuda_stream)
    ctx.step(warmup, use_graph=True)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s)
    ctx.step(steps, use_graph=True)
    e1.record(s)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    n = w.grid.nx * w.grid.ny * w.grid.nz
    um, phi = ctx.download()
    ok = bool(np.isfinite(um).all() and np.isfinite(phi).all())
    dev_bytes = ctx.device_bytes()
    ctx.close()
    return {
        "workload": "stirred tank 512x512x384 walls, RK3 step with WENO5 level set",
        "cells": n, "steps": steps, "value": round(n / (ms * 1e-3) / 1e6, 3),
        "unit": "Mcell-RK3-steps/s", "ms_per_step": round(ms, 3),
        "device_gib": round(dev_bytes / 2**30, 2), "finite": ok,
    }


def adjoint_leg(n: int = 128, nsteps: int = 8, every: int = 0, stream=None, nz=None, fd=True,
                state_fd=False, reps=3):
    """dJ/d(omega, Cs) of the tank objective after nsteps steps on the n^3 tank
    by the hand-written adjoint, its cost against the forward steps, and the
    finite differences it is checked against.  every = 0: every step's tape
    kept from the forward pass (the tapes of 128^3 x 8 steps fit in HBM, so
    nothing is recomputed); every >= 1: checkpoints every `every` steps, each
    step recomputed with its tape in the reverse sweep.  fd: central
    differences with h = 1e-6 and a Richardson pair per parameter (the
    central ones only where reps > 1, i.e. the smaller workload); state_fd:
    the directional derivative of J in a seeded direction of the initial um
    against the adjoint state gradient."""
    import torch
    from emix_gb300 import _lib
    from emix_gb300 import fields as F
    from emix_gb300 import ops
    w = F.stirred_tank(n=n, nz=nz, impeller=True)
    X, Y, Z = w.grid.coords()
    # free surface with a ripple, inside the box
    w.phi = np.ascontiguousarray(Z - 0.8 * 2.0 + 0.02 * np.sin(3 * X) * np.cos(2 * Y))
    del X, Y, Z
    # `every` may be a list of checkpoint intervals, tried in order until the
    # adjoint's arena fits in device memory
    tries = list(every) if isinstance(every, (list, tuple)) else [every]
    r = None
    for k, ev in enumerate(tries):
        try:
            torch.cuda.empty_cache()
            r = ops.TankGradient(w, nsteps, ev, bc_walls=WALLS)
            every = ev
            break
        except _lib.EmixError as e:
            if e.rc != _lib.EMIX_ERR_ALLOC or k + 1 == len(tries):
                raise
    s = stream or torch.cuda.Stream()
    r.ctx.set_stream(s.cuda_stream)
    om, cs = w.impeller.omega, w.cs
    r.run(om, cs)                     # warm-up (graph capture, tables)
    r.adj.backward()
    # forward (with checkpoints) and reverse sweep, `reps` times: the medians
    fw, bw = [], []
    for _ in range(reps):
        t0 = time.perf_counter()
        J = r.run(om, cs)
        t1 = time.perf_counter()
        g = r.adj.backward()
        t2 = time.perf_counter()
        fw.append(t1 - t0)
        bw.append(t2 - t1)
    t_fw, t_bw = float(np.median(fw)), float(np.median(bw))
    state = None
    if state_fd:
        # <dJ/dum0, d> against (J(um0 + e d) - J(um0 - e d)) / 2e
        lum, _ = r.adj.state_gradient()
        lum = lum.cpu().numpy()    # the product on the host: no device memory beside the arenas
        um0 = w.um
        u = F.uniform(93, 0, um0.shape[1:])
        d = np.stack([(1e-2 * (-1.0) ** m * float(np.abs(um0[m]).max())) * u for m in range(5)])
        del u
        pred = float(np.sum(lum * d))
        del lum
        eps = 1e-4
        vals = []
        for sgn in (1.0, -1.0):
            w.um = np.ascontiguousarray(um0 + sgn * eps * d)
            vals.append(r.run(om, cs))
        w.um = um0
        fdv = (vals[0] - vals[1]) / (2 * eps)
        state = {"direction": "1e-2 x (-1)^m x max|um_m| x one seeded uniform field, e = 1e-4",
                 "adjoint": pred, "fd": fdv, "rel_err": abs(pred - fdv) / abs(fdv)}
        del d
    fds, rich = [], []

    def cfd(k, p0, h):
        a = [om, cs]; a[k] = p0 + h
        b = [om, cs]; b[k] = p0 - h
        return (r.run(*a) - r.run(*b)) / (2 * h)

    for k, p0 in enumerate((om, cs) if fd else ()):
        # central differences with h = 1e-6 (rounding-limited when dJ is small
        # against J), and a Richardson pair h, h/2 (error O(h^4))
        if reps > 1:
            fds.append(cfd(k, p0, 1e-6 * max(abs(p0), 1.0)))
        # omega moves the blades: a step small enough that no cell changes side
        h = (1e-3 if k == 0 else 1e-2) * abs(p0)
        rich.append((4.0 * cfd(k, p0, 0.5 * h) - cfd(k, p0, h)) / 3.0)
    # plain steps without checkpoints, for the cost ratio (median of `reps`)
    r.ctx.upload(w.um, w.phi)
    r.ctx.step(1, use_graph=True)
    torch.cuda.synchronize()
    pl = []
    for _ in range(reps):
        t3 = time.perf_counter()
        r.ctx.step(nsteps, use_graph=True)
        torch.cuda.synchronize()
        pl.append(time.perf_counter() - t3)
    gib = r.adj.device_bytes() / 2**30
    ctx_gib = r.ctx.device_bytes() / 2**30
    r.close()
    cells = w.grid.ncell
    plain = float(np.median(pl))
    # for comparison: checkpoints every step, each step recomputed with its tape
    recompute = None
    if every == 0:
        r1 = ops.TankGradient(w, nsteps, 1, bc_walls=WALLS)
        r1.ctx.set_stream(s.cuda_stream)
        r1.run(om, cs)
        r1.adj.backward()
        fw1, bw1 = [], []
        for _ in range(reps):
            t0 = time.perf_counter()
            r1.run(om, cs)
            t1 = time.perf_counter()
            r1.adj.backward()
            t2 = time.perf_counter()
            fw1.append(t1 - t0)
            bw1.append(t2 - t1)
        gib1 = r1.adj.device_bytes() / 2**30
        r1.close()
        f1, b1 = float(np.median(fw1)), float(np.median(bw1))
        recompute = {"checkpoint_every": 1, "forward_s": round(f1, 4), "backward_s": round(b1, 4),
                     "adjoint_over_forward": round(b1 / plain, 3),
                     "gradient_over_forward": round((f1 + b1) / plain, 3), "adjoint_gib": round(gib1, 2)}
    return {
        "workload": f"stirred tank {n}x{n}x{nz or n} walls + rotating impeller, {nsteps} RK3 steps, "
                    "J = annulus kinetic energy + interface area",
        "J": J, "dJ_domega": g[0], "dJ_dCs": g[1],
        "fd_domega": fds[0] if fds else None, "fd_dCs": fds[1] if fds else None,
        "rel_err": [abs(g[0] - fds[0]) / abs(fds[0]), abs(g[1] - fds[1]) / abs(fds[1])] if fds else None,
        "richardson_fd": rich or None,
        "rel_err_richardson": [abs(g[i] - rich[i]) / abs(rich[i]) for i in range(2)] if rich else None,
        "state_direction": state,
        "forward_s": round(t_fw, 4), "backward_s": round(t_bw, 4), "plain_steps_s": round(plain, 4),
        "timing": f"medians of {reps} runs each" if reps > 1 else "one run after a warm-up run",
        "adjoint_over_forward": round(t_bw / plain, 3),
        "gradient_over_forward": round((t_fw + t_bw) / plain, 3),
        "mode": "tapes kept from the forward pass" if every == 0 else f"checkpoints every {every}, recomputed",
        "forward_value": round(cells * nsteps / plain / 1e6, 3),
        "adjoint_value": round(cells * nsteps / t_bw / 1e6, 3),
        "unit": "Mcell-RK3-steps/s", "checkpoint_every": every, "adjoint_gib": round(gib, 2),
        "context_gib": round(ctx_gib, 2),
        "recompute": recompute,
    }


def config_dict(w):
    return {
        "workload": f"stirred tank {N_GRID}^3 walls, RK3 step with WENO5 level set",
        "grid": [N_GRID, N_GRID, N_GRID],
        "scheme": "Lele-6 compact, 3rd/4th-order closures (derivada_incomp.f90)",
        "sgs": "Smagorinsky Cs=0.1", "level_set": "WENO5 TVD stage per substep",
        "walls": "frontera_z/y/x_val after every RK combination" if WALLS else "none",
        "impeller": ("6-blade rotating forcing at z=H/3, blade radius 0.33R, height 0.05H, "
                     "omega=1" if IMPELLER else "static mask"),
        "cfl": 0.3, "dt": None if w is None else w.dt, "precision": "fp64",
        "l2": "inputs larger than L2 (9 GB resident, 128 MiB per field)",
        "parallelism": "replicas (one independent grid per GPU)",
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="emix", choices=["emix", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the batched-ensemble leg")
    ap.add_argument("--no-large", action="store_true", help="skip the 512x512x384 leg")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint (gradient) leg")
    ap.add_argument("--no-large-adjoint", action="store_true",
                    help="skip forward + adjoint on 512x512x384 (20 steps, checkpoints every 5)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import torch.distributed as dist
    from emix_gb300 import fields as F
    from emix_gb300 import ops

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from emix_gb300 import replicas

    def barrier():
        replicas.barrier(world)

    def max_over_ranks(x: float) -> float:
        return replicas.max_over_ranks(x, world, "cuda")

    w = F.stirred_tank(n=N_GRID, impeller=IMPELLER)
    n = w.grid.ncell
    ng = (N_GRID + 2 * G) ** 3
    ctx = ops.Context(w, level_set=True, ls_ghost=G, bc_walls=WALLS)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    ctx.step(args.warmup, use_graph=True)
    torch.cuda.synchronize()

    # ---- device-resident timed region ----
    sampler = ClockSampler(local)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    sampler.start()
    time.sleep(0.3)
    e0.record(stream)
    ctx.step(args.steps, use_graph=True)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    barrier()
    ms = max_over_ranks(e0.elapsed_time(e1))
    value = world * n * args.steps / (ms * 1e-3) / 1e6
    launches_per_step = ctx.launches_per_step()
    # the same steps on one stream (no concurrent launches), for reference
    ctx.set_overlap(0)
    ctx.step(1, use_graph=True)
    g0 = torch.cuda.Event(enable_timing=True)
    g1 = torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    ctx.step(args.steps, use_graph=True)
    g1.record(stream)
    torch.cuda.synchronize()
    ms_one = g0.elapsed_time(g1) / args.steps
    ctx.set_overlap(3)

    # ---- end-to-end through the host-pointer entry point ----
    um_h = torch.from_numpy(np.ascontiguousarray(w.um)).pin_memory()
    phi_h = torch.from_numpy(np.ascontiguousarray(w.phi)).pin_memory()
    um_np, phi_np = um_h.numpy(), phi_h.numpy()
    ctx.step_host(um_np, phi_np, 1)
    torch.cuda.synchronize()
    barrier()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(args.steps):
        ctx.step_host(um_np, phi_np, 1)
    f1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms_e2e = max_over_ranks(f0.elapsed_time(f1))
    e2e_value = world * n * args.steps / (ms_e2e * 1e-3) / 1e6
    assert np.isfinite(um_np).all() and np.isfinite(phi_np).all()
    # the host link this box gives: um's pinned buffer to and from the device
    dev_um = torch.empty(um_h.shape, dtype=um_h.dtype, device="cuda")
    link = {}
    for name, dst, src in (("h2d_gbs", dev_um, um_h), ("d2h_gbs", um_h, dev_um)):
        best = 1e30
        for _ in range(3):
            l0 = torch.cuda.Event(enable_timing=True)
            l1 = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                l0.record(stream)
                dst.copy_(src, non_blocking=True)
                l1.record(stream)
            torch.cuda.synchronize()
            best = min(best, l0.elapsed_time(l1))
        link[name] = round(um_h.numel() * 8 / (best * 1e-3) / 1e9, 1)
    del dev_um

    # ---- per-kernel times (CUDA events around every launch) ----
    prof = ctx.profile(nsteps=max(3, min(args.steps, 10)))
    psteps = max(3, min(args.steps, 10))
    total = sum(v[0] for v in prof.values()) or 1.0
    kernels = {k: {"ms_per_launch": round(v[0] / v[1], 4) if v[1] else 0.0,
                   "launches_per_step": v[1] // psteps,
                   "share": round(v[0] / total, 4)} for k, v in prof.items() if v[1]}
    top = max(prof, key=lambda k: prof[k][0])
    top_ms = prof[top][0] / prof[top][1]
    hbm_peak, peak_kind = _peaks()
    fp64_peak = ops.fp64_peak()
    ab = algorithmic_bytes(top, n, ng, dims=(N_GRID,) * 3, g=G)
    cells_top = cells_per_launch(top, (N_GRID,) * 3, G)
    fp64_ach = FP64_OPS_PER_CELL.get(top, 0) * cells_top / (top_ms * 1e-3)
    achieved = ab / (top_ms * 1e-3) / 1e9
    traffic = DRAM_BYTES_PER_CELL.get(top)
    if traffic is not None:
        traffic = round(traffic * cells_top)
    roofline = {
        "kernel": top, "bound": "hbm", "achieved": round(achieved, 2), "peak": hbm_peak,
        "unit": "GB/s", "frac": round(achieved / hbm_peak, 4), "traffic": traffic,
        "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
        "traffic_source": CONSTANT_SOURCES["dram_bytes_per_cell"],
        "binding": "fp64",
        "fp64": {"achieved": round(fp64_ach / 1e9, 2), "peak": round(fp64_peak / 1e9, 2),
                 "unit": "G FP64 lane-ops/s", "frac": round(fp64_ach / fp64_peak, 4),
                 "peak_source": "measured live (emix_fp64_peak: FMA chains)"},
    }
    # the whole step against the FP64 issue limit and against HBM at the
    # algorithmic floor of 2064 B per cell-step (every field of every
    # substep's kernel contracts read or written once, Smagorinsky)
    ops_step = 0.0
    for k, v in kernels.items():
        cnt = 3 * n if k == "rk_post" else cells_per_launch(k, (N_GRID,) * 3, G) * v["launches_per_step"]
        ops_step += FP64_OPS_PER_CELL.get(k, 0.0) * cnt
    sec_step = ms / args.steps * 1e-3
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    issue = 2.0 * sms * (clocks.get("sm_max_mhz") or 2070.0) * 1e6
    floor_b = 2064.0
    step_roofline = {
        "fp64_ops_per_cell_step": round(ops_step / n, 1),
        "fp64_ops_source": CONSTANT_SOURCES["fp64_ops_per_cell"],
        "fp64_achieved_gops": round(ops_step / sec_step / 1e9, 1),
        "fp64_issue_limit_gops": round(issue / 1e9, 1),
        "fp64_frac_of_issue_limit": round(ops_step / sec_step / issue, 4),
        "hbm_floor_bytes_per_cell_step": floor_b,
        "hbm_achieved_gbs": round(floor_b * n / sec_step / 1e9, 1),
        "hbm_frac": round(floor_b * n / sec_step / 1e9 / hbm_peak, 4),
    }
    ctx.close()

    line = {
        "metric": "Mcell-RK3-steps/s", "value": round(value, 3), "unit": "Mcell-RK3-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms / args.steps, 4), "ms_per_step_one_stream": round(ms_one, 4),
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_dict(w),
        "e2e": {"value": round(e2e_value, 3), "unit": "Mcell-RK3-steps/s",
                "h2d_bytes_per_step": int(6 * n * 8), "d2h_bytes_per_step": int(6 * n * 8),
                "api": "emix_step_host (pinned host buffers, H2D um+phi, one step, D2H um+phi)",
                "host_link": link},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": roofline,
        "step_roofline": step_roofline,
        "kernels": kernels,
        "clocks": {k: clocks[k] for k in ("sm_mhz", "sm_max_mhz", "reasons")},
    }
    # the single-grid side workloads run at N = 1 only (the scaling runs time
    # the headline step); the ensemble splits its grids between the ranks
    if not args.no_ensemble:
        # N = 1: the whole ensemble; N > 1: the grids split between the ranks
        line["ensemble"] = ensemble_leg(min(args.steps, 10), 3, stream, world, rank)
    if world == 1 and not args.no_large:
        line["large"] = large_leg(min(args.steps, 5), 3, stream)
    if world == 1 and not args.no_adjoint:
        line["adjoint"] = adjoint_leg(stream=stream)
    if world == 1 and not args.no_large_adjoint:
        # checkpoints every step where the arena fits (one taped recompute per
        # step in the reverse sweep), else every 2 or 5 steps
        line["large_adjoint"] = adjoint_leg(512, 20, [1, 2, 5], stream, nz=384, fd=True, state_fd=True, reps=1)
    if rank == 0 and world == 1 and not args.no_cpu:
        # all host threads on the headline workload itself (its fields, two
        # steps), and one thread (the reference's serial build) on one step of
        # the 128^3 tank of the same generator
        v, sec, thr = cpu_sample(N_GRID, 2, 0, w=w)
        v1, sec1, _ = cpu_sample(SINGLE_N, 1, 0, threads=1)
        line["cpu_baseline"] = {
            "value": round(v, 4), "unit": "Mcell-RK3-steps/s", "cores": thr, "kind": "port",
            "sample": f"2 RK3 steps of the {N_GRID}^3 stirred tank (the workload of the config), CPU "
                      f"restatement of the reference algorithm, {sec:.1f} s, {thr} threads",
            "single_thread": {"value": round(v1, 4), "unit": "Mcell-RK3-steps/s", "cores": 1,
                              "sample": f"1 RK3 step of the {SINGLE_N}^3 stirred tank (same generator "
                                        f"and settings), {sec1:.1f} s, 1 thread"}}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
