"""Benchmark of the fused D3Q19 hot path on GB300.

Workload (one "step" = one fused LBM time step over the whole grid):
  256 x 128 x 128 cells, sphere r = 0.5 world (D = 32 cells) at the domain
  centre, Re = 100 (U = 0.05, nu = 0.016, tau = 0.548), MRT collision with the
  Smagorinsky model (Cs = 0.1), ray-sphere Bouzidi q on a dist^2 <= r^2 mask,
  Zou-He inlet/outlet, periodic y/z, pre-collision stability guard -- the
  examples/10_cd_convergence.py step at its 256x128x128 resolution plus
  Smagorinsky.  Populations stored in FP32 (the headline) and, as extra
  lines, FP16 / BF16 deviations from the free-stream equilibrium.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Timing: W warm-up steps, then K steps bracketed by barrier + synchronize and
CUDA events on the launching stream; the A/B state (2 x 319 MB) is larger than
L2 (129 MB), so every step reads and writes HBM.  With --gpus N > 1 (torchrun)
each rank runs an independent replica ("replicas only": the path is one
domain per GPU) and rank 0 prints the aggregate.

The reference arm (--impl reference) times the CPU oracle -- the torch-CPU
restatement of jax_lbm (JAX itself is not installed) -- on this host's cores.
"""

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NX, NY, NZ = 256, 128, 128
U = 0.05
RE = 100.0
D_CELLS = 2 * 0.5 * NX / 8.0
NU = U * D_CELLS / RE
TAU = 3.0 * NU + 0.5
CS = 0.1
BYTES_PER_UPDATE = {"fp32": 152, "fp16": 76, "bf16": 76, "fp64": 304}
WORKLOAD = ("D3Q19 MRT+Smagorinsky(Cs=0.1) sphere D=32 Re=100, Bouzidi ray-sphere q, "
            "Zou-He in/out, periodic y/z, pre-collision guard, 256x128x128")


def bench_config(ws):
    """The workload description both arms print (the same dict, so the two
    lines name the same configuration)."""
    return {"workload": WORKLOAD, "grid": [NX, NY, NZ], "storage": "fp32",
            "tau": round(TAU, 6), "l2": "inputs larger than L2 (A/B state 638 MB)",
            "parallelism": "replicas" if ws > 1 else "single GPU"}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _traffic_from_profiles(storage):
    """Per-launch DRAM bytes of the fused step from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "k_step_fp32_256x128x128.traffic.json")) as fh:
            d = json.load(fh)
        return d.get(storage)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm, mx, pw = float(p[1]), float(p[2]), float(p[3])
            except ValueError:
                continue
            rows.append((sm, pw, [nm for nm, v in zip(names, p[5:9]) if v.lower() == "active"]))
        if not rows:
            return None
        # under load: samples drawing at least 30 % of the highest power seen
        pmax = max(r[1] for r in rows)
        load = [r for r in rows if r[1] >= 0.3 * pmax] or rows
        for r in load:
            reasons.update(r[2])
        sm = sorted(r[0] for r in load)
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(rows), "samples_under_load": len(load),
                "power_w_max": pmax, "window": "whole bench arm, sampled every 100 ms"}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _oracle_step_sample(n_steps, threads):
    """Time n_steps of the CPU oracle on the bench workload; returns (s, cells*steps)."""
    import torch

    from oracle import drivers, geometry, ops
    torch.set_num_threads(threads)
    solid, q = geometry.create_sphere(NX, NY, NZ, (0.0, 0.0, 0.0), 0.5)
    f = drivers.initial_state(NX, NY, NZ, U)
    cfg = drivers.StepConfig(tau=TAU, inlet=(U, 0.0, 0.0), collision="mrt", smagorinsky_cs=CS,
                             guard="pre")
    with torch.no_grad():
        drivers.step(f, q, cfg, solid=solid, f_ref=f)      # warm-up (allocator, threads)
        t0 = time.perf_counter()
        g = f
        for _ in range(n_steps):
            g, _, _ = drivers.step(g, q, cfg, solid=solid, f_ref=f)
        dt = time.perf_counter() - t0
    return dt, NX * NY * NZ * n_steps


def _oracle_slab(planes, threads):
    """An x-slab of `planes` planes of the bench workload for the CPU oracle:
    the full-grid sphere geometry and initial state cut to x < planes (the
    slab's first and last planes take the inlet / outlet rules)."""
    import torch

    from oracle import drivers, geometry
    torch.set_num_threads(threads)
    solid, q = geometry.create_sphere(NX, NY, NZ, (0.0, 0.0, 0.0), 0.5)
    f = drivers.initial_state(NX, NY, NZ, U)
    x0 = max(0, NX // 2 - planes // 2)
    sl = slice(x0, x0 + planes)
    cfg = drivers.StepConfig(tau=TAU, inlet=(U, 0.0, 0.0), collision="mrt", smagorinsky_cs=CS,
                             guard="pre")
    return (f[:, sl].contiguous(), q[:, sl].contiguous(), solid[sl].contiguous(), cfg)


def run_reference(args):
    """The CPU reference arm: W warm-up and K timed steps of the torch-CPU
    restatement of jax_lbm on all host cores.  Each step is a bounded sample
    of the workload -- one step on an x-slab of the 256x128x128 grid, the
    slab sized from a calibration step so the whole run takes about 90 s."""
    import torch

    from oracle import drivers
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    # calibrate: seconds per plane on a 32-plane slab (larger than the caches)
    f, q, solid, cfg = _oracle_slab(32, threads)
    with torch.no_grad():
        drivers.step(f, q, cfg, solid=solid, f_ref=f)
        t0 = time.perf_counter()
        drivers.step(f, q, cfg, solid=solid, f_ref=f)
        per_plane = (time.perf_counter() - t0) / 32
    budget = 0.8 * 90.0 / (args.steps + args.warmup)
    planes = int(min(NX, max(4, budget / per_plane)))
    f, q, solid, cfg = _oracle_slab(planes, threads)
    with torch.no_grad():
        g = f
        for _ in range(args.warmup):
            g, _, _ = drivers.step(g, q, cfg, solid=solid, f_ref=f)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            g, _, _ = drivers.step(g, q, cfg, solid=solid, f_ref=f)
        dt = time.perf_counter() - t0
    cells = planes * NY * NZ
    mlups = cells * args.steps / dt / 1e6
    sample = ("per step: one step of an x-slab of %d of the 256 planes of the 256x128x128 "
              "workload (%d cells) on the torch-CPU restatement of jax_lbm, %d threads"
              % (planes, cells, threads))
    line = {
        "impl": "reference",
        "metric": "fwd MLUPS at 256x128x128 (MRT+Smagorinsky sphere step)",
        "value": round(mlups, 4), "unit": "MLUPS", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * dt / args.steps * NX / planes, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": bench_config(ws),
        "cpu_baseline": {"value": round(mlups, 4), "unit": "MLUPS", "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(mlups, 4), "unit": "MLUPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def _make_sim(storage):
    from lbm_jax_autodiff_gb300 import Simulation
    sim = Simulation(NX, NY, NZ, TAU, collision="mrt", storage=storage, use_smagorinsky=True,
                     smagorinsky_cs=CS, periodic_yz=True, guard="pre",
                     inlet_velocity=(U, 0.0, 0.0))
    sim.set_sphere(0.5, center=(0.0, 0.0, 0.0), kind="dist", q_mode="bouzidi", porosity="hard")
    sim.set_state(sim.equilibrium_state())
    return sim


def _time_steps(sim, steps, warmup, barrier):
    import torch
    sim.run(warmup)
    torch.cuda.synchronize()
    barrier()
    st = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    sim.run(steps)
    e1.record(st)
    torch.cuda.synchronize()
    barrier()
    return e0.elapsed_time(e1) / 1e3


def _state_api_rate(n_steps=200):
    """The reference-shaped functional API (state.py step / simulate) on the
    bench workload in FP32 with the post-BC guard (state.py:161-169): us per
    step of one simulate(state, params, n) call and of a loop of step()
    calls, beside Simulation.run on the same handle parameters.  Each step()
    returns the reference f: the launch that writes it also performs the next
    step (lbm_get_state_and_step), reading the state once."""
    import torch
    from lbm_jax_autodiff_gb300 import Simulation
    from lbm_jax_autodiff_gb300.geometry.primitives import create_sphere
    from lbm_jax_autodiff_gb300.state import LBMParams, LBMState, clear_handles, simulate, step
    solid, q = create_sphere(NX, NY, NZ, (0.0, 0.0, 0.0), 0.5)
    solid = solid.to(torch.int32)
    sim = Simulation(NX, NY, NZ, TAU, collision="mrt", use_smagorinsky=True, smagorinsky_cs=CS,
                     periodic_yz=True, guard="post", inlet_velocity=(U, 0.0, 0.0))
    sim.set_mask(solid, q=q)
    f0 = sim.equilibrium_state().cuda()
    sim.set_state(f0)

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / n_steps * 1e6

    sim.run(10)
    t_run = timed(lambda: sim.run(n_steps))
    sim.close()
    params = LBMParams(tau=TAU, inlet_velocity=(U, 0.0, 0.0), collision_mode=1,
                       use_smagorinsky=1, smagorinsky_cs=CS, periodic_yz=True)
    state = LBMState(f=f0, solid=solid, q=q)
    simulate(state, params, 10)                    # handle and geometry built once

    def loop():
        st = state
        for _ in range(n_steps):
            st = step(st, params)

    t_sim = timed(lambda: simulate(state, params, n_steps))
    t_step = timed(loop)
    clear_handles()                                # its device memory back for the next lines
    torch.cuda.empty_cache()
    return {"steps": n_steps, "run_us_per_step": round(t_run, 2),
            "simulate_us_per_step": round(t_sim, 2), "step_loop_us_per_step": round(t_step, 2),
            "simulate_over_run": round(t_sim / t_run, 3), "step_loop_over_run": round(t_step / t_run, 3),
            "note": "host wall time; each step() call returns the reference f, written by the "
                    "launch that also performs the next step (152 + 76 B per cell), "
                    "simulate() returns it once per call"}


def _grad_rate(storage, n_steps, reps, barrier, max_over_ranks, peak, ws):
    """dCd/dr (bouzidi_hard sphere, MRT + Smagorinsky, no guard) over n_steps:
    forward with checkpoints, recompute, adjoint; workspace sized to free HBM."""
    import torch
    from lbm_jax_autodiff_gb300 import Simulation
    sim = Simulation(NX, NY, NZ, TAU, collision="mrt", storage=storage, use_smagorinsky=True,
                     smagorinsky_cs=CS, periodic_yz=True, guard="off",
                     inlet_velocity=(U, 0.0, 0.0))
    sim.set_sphere(0.5, center=(0.0, 0.0, 0.0), kind="dist", q_mode="bouzidi", porosity="hard")
    sim.set_state(sim.equilibrium_state())
    cd, g = sim.cd_and_grad(n_steps, checkpoint_every=0)      # warm-up, allocates
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(reps):
        cd, g = sim.cd_and_grad(n_steps, checkpoint_every=0)
    t = max_over_ranks((time.perf_counter() - t0) / reps)
    K, recompute, wbytes = sim.adjoint_plan
    sim.close()
    torch.cuda.empty_cache()
    n_cells = NX * NY * NZ
    bf = BYTES_PER_UPDATE[storage] / 2          # one population pass, bytes per cell
    bl = 8.0 if storage == "fp64" else 4.0      # adjoint state in the compute type
    per_cell = (n_steps * 2 * bf + recompute * 2 * bf + n_steps * (bf + 19 * bl * 2))
    achieved = per_cell * n_cells / t / 1e9
    return {"evals_per_s": round(ws / t, 4), "s_per_eval": round(t, 4), "steps": n_steps,
            "cd": cd, "dcd_dr": g, "segment_steps": K, "recomputed_steps": recompute,
            "workspace_gb": round(wbytes / 1e9, 1),
            "algorithmic_bytes_per_cell_eval": per_cell,
            "achieved_gbs": round(achieved, 1), "frac": round(achieved / peak, 4)}


def _cd_time_average(storage, n_steps, smagorinsky, sample_every=500, tail_fraction=0.3):
    """Cd sampled every `sample_every` steps over n_steps of the sphere at
    256x128x128 (D = 32, Re 100, pre-collision guard), averaged over the last
    30 % of the samples as examples/10_cd_convergence.py:88-106 does
    (n_tail = max(3, int(0.3 n_samples)), mean and population std)."""
    import torch
    from lbm_jax_autodiff_gb300 import Simulation
    sim = Simulation(NX, NY, NZ, TAU, collision="mrt", storage=storage,
                     use_smagorinsky=smagorinsky, smagorinsky_cs=CS, periodic_yz=True,
                     guard="pre", inlet_velocity=(U, 0.0, 0.0))
    sim.set_sphere(0.5, center=(0.0, 0.0, 0.0), kind="dist", q_mode="bouzidi", porosity="hard")
    sim.set_state(sim.equilibrium_state())
    t0 = time.perf_counter()
    smp = sim.run(n_steps, sample_every=sample_every)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    resets = sim.guard_resets
    sim.close()
    cd = smp[:, 3].double().cpu()
    n_tail = max(3, int(cd.numel() * tail_fraction))
    tail = cd[-n_tail:]
    return {"cd_mean": float(tail.mean()), "cd_std": float(tail.std(unbiased=False)),
            "cd_last": float(cd[-1]), "samples": int(cd.numel()), "tail_samples": n_tail,
            "seconds": round(dt, 2), "guard_resets": int(resets)}


def _precision_28k(n_steps):
    """The precision form: the 256x128x128 sphere over n_steps (28,000),
    time-averaged Cd in FP32, FP16, BF16 and FP64 storage with Smagorinsky
    Cs 0.1, each against FP64; and the examples/10 run (MRT without
    Smagorinsky) in the same four storages, each against its FP64 run and
    against the published A100 result 1.1854 +/- 0.0705
    (paper/make_convergence_figures.py:53-54)."""
    out = {"steps": n_steps, "sample_every": 500}
    smag = {}
    for storage in ("fp64", "fp32", "fp16", "bf16"):
        smag[storage] = _cd_time_average(storage, n_steps, True)
    ref = smag["fp64"]["cd_mean"]
    for storage in ("fp32", "fp16", "bf16"):
        smag[storage]["cd_mean_rel_err_vs_fp64"] = abs(smag[storage]["cd_mean"] - ref) / abs(ref)
    out["smagorinsky_cs0.1"] = smag
    pub_mean, pub_std = 1.1854, 0.0705
    ex10 = {}
    for storage in ("fp64", "fp32", "fp16", "bf16"):
        r = _cd_time_average(storage, n_steps, False)
        r["published_cd_mean"], r["published_cd_std"] = pub_mean, pub_std
        r["deviation_in_published_std"] = (r["cd_mean"] - pub_mean) / pub_std
        ex10[storage] = r
    ref = ex10["fp64"]["cd_mean"]
    for storage in ("fp32", "fp16", "bf16"):
        ex10[storage]["cd_mean_rel_err_vs_fp64"] = abs(ex10[storage]["cd_mean"] - ref) / abs(ref)
    out["examples10_no_smagorinsky"] = ex10
    return out


def _batch_rate(n_steps, barrier, max_over_ranks):
    """The batched workload: 64 sphere instances (grids 64x32x32 / 96x48x48 /
    128x64x64, radii, q and porosity modes and alpha drawn with seed 0), MRT
    FP32; one optimisation iteration = n_steps forward + recompute + adjoint of
    every instance and one Adam step on every radius, replayed as one CUDA
    graph (the host rebuilds the geometry of the new radii afterwards, inside
    the timed region)."""
    import torch
    from lbm_jax_autodiff_gb300.batch import Batch, mixed_sphere_instances
    inst, sph = mixed_sphere_instances()
    b = Batch(inst)
    b.set_spheres(sph)
    b.set_equilibrium()
    t0 = time.perf_counter()
    block, K = b.autotune(8, n_steps)
    t_tune = time.perf_counter() - t0
    kw = dict(lr=0.05, r_min=0.3, r_max=1.2, checkpoint_every=K, use_graph=True)
    h0 = b.optimize(1, n_steps, **kw)            # captures the graph and runs it once
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    h1 = b.optimize(1, n_steps, **kw)            # graph replay
    t = max_over_ranks(time.perf_counter() - t0)
    blk, seg, rec, wbytes, graph_s = b.plan
    launches = b.graph_launches
    cells = b.cells
    b.close()
    torch.cuda.empty_cache()
    # error against FP64 storage: the first n_check instances (both q modes,
    # both porosity modes) re-evaluated alone in FP64 at the radius the timed
    # iteration evaluated
    from lbm_jax_autodiff_gb300 import Simulation
    n_check = min(8, len(inst))
    cd_err, g_err = [], []
    for i in range(n_check):
        p = dict(inst[i])
        p["storage"] = "fp64"
        nx, ny, nz = p.pop("nx"), p.pop("ny"), p.pop("nz")
        tau = p.pop("tau")
        s64 = Simulation(nx, ny, nz, tau, **p)
        s64.set_sphere(**dict(sph[i], radius=float(h1["r"][0][i])))
        s64.set_state(s64.equilibrium_state())
        cd64, g64 = s64.cd_and_grad(n_steps, checkpoint_every=0)
        s64.close()
        cd_err.append(abs(float(h1["cd"][0][i]) - cd64) / abs(cd64))
        if g64 != 0.0:
            g_err.append(abs(float(h1["grad"][0][i]) - g64) / abs(g64))
        else:
            g_err.append(0.0 if float(h1["grad"][0][i]) == 0.0 else float("inf"))
    torch.cuda.empty_cache()
    return {"instances": len(inst), "cells": cells, "block": blk, "segment_steps": seg,
            "cd_rel_err_vs_fp64_max": max(cd_err), "grad_rel_err_vs_fp64_max": max(g_err),
            "fp64_checked_instances": n_check,
            "recomputed_steps": rec, "workspace_gb": round(wbytes / 1e9, 1),
            "autotune_s": round(t_tune, 2), "graph_capture_s": round(graph_s, 3),
            "graph_kernel_launches": launches, "s_per_iter": round(t, 3),
            "instance_grads_per_s": round(len(inst) / t, 2),
            "cell_steps_per_s_M": round(cells * (2 * n_steps + rec) / t / 1e6, 1),
            "cd_mean": round(float(h1["cd"][0].mean()), 6),
            "mean_abs_dr": round(float(abs(h1["r_final"] - h0["r_final"]).mean()), 6),
            "note": "per iteration: %d forward + %d recompute + %d adjoint batched launches over "
                    "all instances, Adam (lr 0.05, clip [0.3, 1.2]) on the device, geometry "
                    "rebuild on the host" % (n_steps, rec, n_steps)}


def rank_ops(dist, device):
    """(barrier, max_over_ranks) over an initialised process group; dist None
    for one rank.  Every timed figure is the maximum over ranks."""
    import torch

    def barrier():
        if dist is not None:
            dist.barrier()

    def max_over_ranks(v):
        if dist is None:
            return v
        t = torch.tensor([v], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    return barrier, max_over_ranks


def aggregate_mlups(ws, cells, steps, seconds):
    """Whole-job MLUPS: every rank advances its own replica of `cells` cells."""
    return ws * cells * steps / seconds / 1e6


def run_ours(args):
    import torch
    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    barrier, max_over_ranks = rank_ops(dist, "cuda")

    n_cells = NX * NY * NZ
    peak, peak_kind = _peaks()

    # clocks and throttle reasons over the whole arm (the headline's timed
    # region alone is a few ms, shorter than the sampling interval)
    clocks = ClockSampler(local)
    clocks.start()

    # headline: FP32 storage
    sim = _make_sim("fp32")
    t = _time_steps(sim, args.steps, args.warmup, barrier)
    t = max_over_ranks(t)
    mlups = aggregate_mlups(ws, n_cells, args.steps, t)
    per_launch = t / args.steps
    achieved = BYTES_PER_UPDATE["fp32"] * n_cells / per_launch / 1e9

    # e2e through the public API with host buffers (pinned), chunks of 500
    # steps -- the reference drivers' sampling interval (examples/10:93-97):
    # each chunk copies its input state in from the host, runs the steps
    # with the Cd sampled after the last one, and copies the state and the
    # Cd back.  The copies of a chunk overlap the previous / next chunk's
    # steps on a second stream (double-buffered device staging), as a
    # pipelined driver would do; one serialised chunk, timed by phase with
    # CUDA events, shows what each copy costs.
    chunk = 500
    n_chunks = max(4, args.steps // chunk)
    f_host = sim.equilibrium_state().cpu().pin_memory()
    f_out = [torch.empty_like(f_host).pin_memory() for _ in range(2)]
    cd_host = [torch.empty((1, 4), dtype=torch.float64).pin_memory() for _ in range(2)]
    samples = [torch.zeros((1, 4), dtype=torch.float64, device="cuda") for _ in range(2)]
    d_in = [torch.empty_like(f_host, device="cuda") for _ in range(2)]
    d_out = [torch.empty_like(f_host, device="cuda") for _ in range(2)]
    main = torch.cuda.current_stream()
    side = torch.cuda.Stream()

    def ev():
        return torch.cuda.Event()

    def e2e_pipelined(n):
        in_ready, in_used, out_ready, out_free = ([ev(), ev()] for _ in range(4))
        for b in range(2):
            in_used[b].record(main)
            out_free[b].record(main)
        with torch.cuda.stream(side):
            d_in[0].copy_(f_host, non_blocking=True)
            in_ready[0].record(side)
        for i in range(n):
            b = i % 2
            if i + 1 < n:
                side.wait_event(in_used[1 - b])
                with torch.cuda.stream(side):
                    d_in[1 - b].copy_(f_host, non_blocking=True)
                    in_ready[1 - b].record(side)
            main.wait_event(in_ready[b])
            sim.set_state(d_in[b])
            in_used[b].record(main)
            sim.run(chunk, sample_every=chunk, samples=samples[b])
            main.wait_event(out_free[b])
            sim.get_state(out=d_out[b])
            out_ready[b].record(main)
            side.wait_event(out_ready[b])
            with torch.cuda.stream(side):
                f_out[b].copy_(d_out[b], non_blocking=True)
                cd_host[b].copy_(samples[b], non_blocking=True)
                out_free[b].record(side)
        torch.cuda.synchronize()

    # serialised chunk, by phase
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
    e2e_pipelined(1)                       # first touch of the pinned pages (~250 ms once)
    evs[0].record(main)
    sim.set_state_host(f_host)
    evs[1].record(main)
    sim.run(chunk, sample_every=chunk, samples=samples[0])
    evs[2].record(main)
    sim.get_state_host(f_out[0])
    evs[3].record(main)
    cd_host[0].copy_(samples[0], non_blocking=True)
    evs[4].record(main)
    torch.cuda.synchronize()
    per = [evs[k].elapsed_time(evs[k + 1]) for k in range(4)]
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_pipelined(n_chunks)
    t_e2e = max_over_ranks(time.perf_counter() - t0)
    e2e_mlups = aggregate_mlups(ws, n_cells, chunk * n_chunks, t_e2e)
    state_bytes = 19 * n_cells * 4
    cd_last = float(cd_host[(n_chunks - 1) % 2][0, 3])
    sim.close()
    e2e_note = ("public API (set_state, run, get_state), pinned host state in and out and the Cd "
                "read back every %d-step chunk, the copies overlapping the neighbouring chunks' "
                "steps on a second stream; %d timed chunks, host wall %.2f ms per chunk.  One "
                "serialised chunk (set_state_host, run, get_state_host, Cd): H2D %.2f ms, %d "
                "steps + final Cd sample pass %.2f ms, D2H %.2f ms, Cd read %.3f ms"
                % (chunk, n_chunks, 1e3 * t_e2e / n_chunks, per[0], chunk, per[1], per[2],
                   per[3]))

    # secondary lines: 16-bit storage of f - f_eq(1, U)
    extra = {}
    for storage in ("fp16", "bf16"):
        s2 = _make_sim(storage)
        t2 = max_over_ranks(_time_steps(s2, args.steps, args.warmup, barrier))
        s2.close()
        extra[storage] = {
            "mlups": round(aggregate_mlups(ws, n_cells, args.steps, t2), 1),
            "achieved_gbs": round(BYTES_PER_UPDATE[storage] * n_cells / (t2 / args.steps) / 1e9, 1),
            "frac": round(BYTES_PER_UPDATE[storage] * n_cells / (t2 / args.steps) / 1e9 / peak, 4),
        }

    # in-place (AA) streaming of the FP32 step: one population buffer instead of two
    s3 = _make_sim("fp32")
    s3.set_streaming("aa")
    t3 = max_over_ranks(_time_steps(s3, args.steps, args.warmup, barrier))
    s3.close()
    extra["fp32_inplace"] = {
        "mlups": round(aggregate_mlups(ws, n_cells, args.steps, t3), 1),
        "achieved_gbs": round(BYTES_PER_UPDATE["fp32"] * n_cells / (t3 / args.steps) / 1e9, 1),
        "frac": round(BYTES_PER_UPDATE["fp32"] * n_cells / (t3 / args.steps) / 1e9 / peak, 4),
        "population_buffers": 1,
        "note": "lbm_set_streaming(LBM_STREAM_AA): one 319 MB state buffer (two for the headline)",
    }

    # the reference-shaped functional API (step / simulate) on the same workload
    state_api = _state_api_rate()

    # shape gradient: dCd/dr evaluations per second over a 2000-step window
    grad = {}
    if not args.no_grad:
        for storage in ("fp32", "fp16", "bf16"):
            grad[storage] = _grad_rate(storage, args.grad_steps, args.grad_reps, barrier,
                                       max_over_ranks, peak, ws)
        if grad["fp32"]["evals_per_s"] > 0:
            grad["fp16_over_fp32"] = round(grad["fp16"]["evals_per_s"] /
                                           grad["fp32"]["evals_per_s"], 3)
        # FP64-storage oracle of the same evaluation; errors of every form against it
        ref = _grad_rate("fp64", args.grad_steps, 1, barrier, max_over_ranks, peak, ws)
        grad["fp64"] = ref
        for storage in ("fp32", "fp16", "bf16"):
            grad[storage]["cd_rel_err_vs_fp64"] = abs(grad[storage]["cd"] - ref["cd"]) / abs(ref["cd"])
            grad[storage]["grad_rel_err_vs_fp64"] = (abs(grad[storage]["dcd_dr"] - ref["dcd_dr"]) /
                                                     abs(ref["dcd_dr"]))

    batch = None
    if not args.no_batch:
        batch = _batch_rate(args.grad_steps, barrier, max_over_ranks)

    precision = None
    if args.cd_steps > 0:
        precision = _precision_28k(args.cd_steps)

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        steps_cpu = max(1, args.steps_ref)
        dt, updates = _oracle_step_sample(steps_cpu, threads)
        cpu = {"value": round(updates / dt / 1e6, 4), "unit": "MLUPS", "cores": threads,
               "kind": "port",
               "sample": "%d step(s) of the full 256x128x128 workload on the torch-CPU "
                         "restatement of jax_lbm (%d threads)" % (steps_cpu, threads)}

    clk = clocks.stop()
    if rank == 0:
        line = {
            "metric": "fwd MLUPS at 256x128x128 (MRT+Smagorinsky sphere step)",
            "value": round(mlups, 1), "unit": "MLUPS", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1e3 * t / args.steps, 5),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": bench_config(ws),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "peak_kind": peak_kind,
                         "traffic": _traffic_from_profiles("fp32"),
                         "algorithmic_bytes_per_update": BYTES_PER_UPDATE["fp32"]},
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e_mlups, 1), "unit": "MLUPS",
                    "h2d_bytes_per_step": state_bytes // chunk,
                    "d2h_bytes_per_step": (state_bytes + 32) // chunk,
                    "serialised_chunk_ms": {"h2d": round(per[0], 3), "run": round(per[1], 3),
                                            "d2h": round(per[2], 3), "cd": round(per[3], 4)},
                    "note": e2e_note},
            "gpu_launches": args.steps,
            "clocks": clk,
            "storage16": extra,
            "grad": grad,
            "batch": batch,
            "precision_28k": precision,
            "state_api": state_api,
            "cd_last_sample": cd_last,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_profile_case(spec):
    """A small fixed workload for ncu captures of one kernel family (no
    timing, no JSON line):

      NXxNYxNZ:STORAGE:STEPS[:grad|:aa]  the bench step (MRT + Smagorinsky
          Cs 0.1, pre-collision guard, dist-mask Bouzidi sphere r = 0.5 world
          at the domain centre, Re 100 on D = nx/8) for STEPS steps; with
          ``grad`` one dCd/dr evaluation over STEPS steps instead (guard off,
          segment STEPS/4: forward, recompute and adjoint kernels); with ``aa``
          the steps run with in-place streaming (k_step_aa);
      batch:COUNT:STEPS  one batched gradient evaluation (no graph) of the
          first COUNT instances of the batched workload, segment STEPS/2.
    """
    import torch
    parts = spec.split(":")
    if parts[0] == "batch":
        from lbm_jax_autodiff_gb300.batch import Batch, mixed_sphere_instances
        count = int(parts[1]) if len(parts) > 1 else 16
        steps = int(parts[2]) if len(parts) > 2 else 8
        inst, sph = mixed_sphere_instances(count)
        b = Batch(inst)
        b.set_spheres(sph)
        b.set_equilibrium()
        cd, g = b.cd_and_grad(steps, checkpoint_every=max(1, steps // 2), use_graph=False)
        torch.cuda.synchronize()
        print("profile case ok: cells", b.cells, "cd[:2]", cd[:2], "g[:2]", g[:2])
        b.close()
        return 0
    from lbm_jax_autodiff_gb300 import Simulation
    nx, ny, nz = [int(v) for v in parts[0].split("x")]
    storage = parts[1] if len(parts) > 1 else "fp32"
    steps = int(parts[2]) if len(parts) > 2 else 8
    grad = len(parts) > 3 and parts[3] == "grad"
    aa = len(parts) > 3 and parts[3] == "aa"
    tau = 3 * U * (nx / 8.0) / RE + 0.5
    sim = Simulation(nx, ny, nz, tau, collision="mrt", storage=storage, use_smagorinsky=True,
                     smagorinsky_cs=CS, guard="off" if grad else "pre",
                     inlet_velocity=(U, 0.0, 0.0))
    sim.set_sphere(0.5, kind="dist", q_mode="bouzidi", porosity="hard")
    if aa:
        sim.set_streaming("aa")
    sim.set_state(sim.equilibrium_state())
    if grad:
        cd, g = sim.cd_and_grad(steps, checkpoint_every=max(1, steps // 4))
        print("cd", cd, "dcd_dr", g)
    else:
        sim.run(steps)
    torch.cuda.synchronize()
    print("profile case ok: links", sim.link_count)
    sim.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--steps-ref", type=int, default=3, help="oracle steps in the CPU sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-grad", action="store_true", help="skip the dCd/dr measurement")
    ap.add_argument("--grad-steps", type=int, default=2000)
    ap.add_argument("--grad-reps", type=int, default=2)
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-instances line")
    ap.add_argument("--cd-steps", type=int, default=28000,
                    help="steps of the time-averaged Cd runs of the precision form (0: skip)")
    ap.add_argument("--profile-case", default=None,
                    help="run a small fixed workload for an ncu capture instead of the bench "
                         "(NXxNYxNZ:STORAGE:STEPS[:grad] or batch:COUNT:STEPS)")
    args = ap.parse_args()
    if args.profile_case:
        return run_profile_case(args.profile_case)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
