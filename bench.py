#!/usr/bin/env python3
"""Benchmark of the GB300 SPH step: particle-updates/s on the 1,048,576-particle dam break.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = grid rebuild + density/pressure + force/integrate over all particles
(the reference's three dispatches, Main.cpp:291-304). The timed region is K steps of
the dam break after W warm-up steps from its initial state; every step is timed with
CUDA events on the simulation stream and L2 is flushed (256 MiB write) between steps,
outside the events. Prints one JSON line (rank 0).

--impl reference times the CPU implementation of the same step on the host cores: the
FP64 restatement of the reference shaders (oracle/), grid back-end, all host threads, on
the same 1,048,576-particle dam break over the same steps (W warm-up steps, then the first
min(K, 30) of the K steps the GPU arm times). It loads nothing but oracle/.
For N > 1 every rank advances its own replica (the path does not shard: "replicas only").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path[:0] = [str(REPO / "npr-sph_gb300"), str(REPO)]

METRIC = "SPH particle-updates/s at 1M on 1 GB300: learned vs plain at <=1% density err"
UNIT = "particle-updates/s"
# Algorithmic HBM bytes per particle-update (each particle's data leaves HBM once per pass):
#   sort (read pos, vel; write sorted pos, vel)          64
#   density (read pos; write rho, p)                     24
#   force+integrate (read pos, vel, rho, p; write pos, vel) 72
B_ALG = {"sort": 64, "density": 24, "force_integrate": 72}
B_ALG_STEP = sum(B_ALG.values())
KERNELS_PER_STEP = 6  # scan_tiles, scan_apply, scatter, gather, density, force_integrate
L2_FLUSH_BYTES = 256 << 20


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(value: float, world: int) -> float:
    """Max of a per-rank float over all ranks (identity for one rank)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


PROFILE = "profiles/pair_kernels_dam_break_1m.md"


def profiled_traffic(kernel: str):
    """DRAM bytes (read + write) per launch of `kernel` from the committed ncu summary of the
    dam break (a line `traffic_bytes_per_launch <kernel>: <bytes>`), or None. ncu cannot run
    inside the timed process, so this figure comes from that capture, not from this run."""
    import re

    prof = REPO / PROFILE
    if not prof.exists():
        return None
    m = re.search(rf"^traffic_bytes_per_launch {re.escape(kernel)}: (\d+)", prof.read_text(), re.M)
    return int(m.group(1)) if m else None


def measured_peaks() -> tuple[dict, str]:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text()), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ["clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.hw_slowdown",
              "clocks_event_reasons.hw_thermal_slowdown", "clocks_event_reasons.sw_thermal_slowdown",
              "clocks_event_reasons.sw_power_cap"]

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={','.join(self.FIELDS)}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) != len(self.FIELDS):
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


CPU_STEPS_MAX = 30  # CPU legs: at most this many timed steps (~0.1 s each at 1M on 16 cores)


def cpu_oracle_legs(warmup: int, steps: int) -> dict:
    """The FP64 oracle (grid back-end, OpenMP, all host threads) on the host cores, on the GPU
    arm's own workloads, loading nothing but oracle/:
      - the 1,048,576-particle dam break (seed 2, as rank 0's GPU replica), W warm-up steps,
        then min(K, 30) timed steps: the first steps of the GPU arm's timed region;
      - the 10,000-particle reference-box scene (config 1): its 200 steps from the start."""
    from oracle import oracle as O
    from oracle import scenes as OS

    params, parts = OS.dam_break(seed=2)
    n = len(parts)
    pos = np.ascontiguousarray(parts["pos"][:, :3], dtype=np.float64)
    vel = np.ascontiguousarray(parts["vel"][:, :3], dtype=np.float64)
    O.run_f64(params, pos, vel, warmup, backend="grid")
    k = max(1, min(steps, CPU_STEPS_MAX))
    t0 = time.perf_counter()
    O.run_f64(params, pos, vel, k, backend="grid")
    el = time.perf_counter() - t0
    p10, s10 = OS.reference_scene_10k(seed=1)
    pos10 = np.ascontiguousarray(s10["pos"][:, :3], dtype=np.float64)
    vel10 = np.ascontiguousarray(s10["vel"][:, :3], dtype=np.float64)
    t1 = time.perf_counter()
    O.run_f64(p10, pos10, vel10, 200, backend="grid")
    el10 = time.perf_counter() - t1
    cores = O.max_threads()
    return {"value": n * k / el, "unit": UNIT, "cores": cores, "kind": "port", "model": OS.cpu_model(),
            "particles": n, "steps": k, "ms_per_step": 1e3 * el / k,
            "sample": f"FP64 oracle (grid back-end, OpenMP, {cores} threads) on the 1,048,576-particle dam break: "
                      f"steps {warmup + 1}-{warmup + k}, the first {k} of the GPU arm's timed steps, {el:.1f} s",
            "reference_scene_10k": {"value": len(s10) * 200 / el10, "unit": UNIT, "particles": len(s10),
                                    "steps": 200, "ms_per_step": 1e3 * el10 / 200,
                                    "workload": "config 1: 10,000 particles at 0.5h in the lower-corner quarter "
                                                "of the reference box, 200 steps from the start"}}


def run_reference(args) -> None:
    """CPU implementation of the step (the FP64 restatement of the reference shaders) on the
    host cores, on the GPU arm's workload and steps."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    leg = cpu_oracle_legs(args.warmup, args.steps)
    v = leg["value"]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": leg["steps"], "warmup": args.warmup, "ms_per_step": leg["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "particles": leg["particles"],
                       "timed_steps": [args.warmup, args.warmup + leg["steps"]],
                       "sample": f"the first {leg['steps']} of the {args.steps} steps the GPU arm times"},
            "cpu_baseline": leg,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)


WORKLOAD = ("dam break: 1,048,576 particles (64x128x128 block, 0.5h lattice, jitter 0.01h) against the x=0 wall "
            "of a 5.12x1.28x1.28 box, g=-9.81, dt=1e-4, plain SPH")


def timed_steps(sim, stream, steps: int, warmup: int) -> float:
    """Seconds of `steps` sph_step calls after `warmup`, by CUDA events on the simulation stream."""
    import torch

    sim.step(warmup)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    sim.step(steps)
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / 1e3


def extra_workloads(args, stream) -> dict:
    """The other two plain configurations, measured the same way (no L2 flush: the batched
    state, ~4.7M particles, is larger than L2; the 10k scene is launch-bound)."""
    import nprsph as S

    out = {}
    plist, counts, parts = S.batched_scenes(256, seed=3)
    n = int(counts.sum())
    with S.Sim(plist, counts=counts, stream=stream.cuda_stream) as sim:
        sim.upload(parts)
        ms = sim.autotune(3) if args.autotune else None
        sim.upload(parts)
        sec = timed_steps(sim, stream, args.extra_steps, 5)
        fb = sim.tile_stats()
        out["batched_256_scenes"] = {
            "value": n * args.extra_steps / sec, "unit": UNIT, "particles": n, "scenes": 256, "steps": args.extra_steps,
            "ms_per_step": 1e3 * sec / args.extra_steps, "launch": list(sim.get_launch()),
            "global_path_chunks": list(fb), "autotune_ms": ms,
            "workload": "256 boxes, counts log-uniform in [2000, 65536], k ~ U[500,3000], mu ~ U[0.1,2], lattice "
                        "or sphere drop; one launch per pass over all scenes, replayed from a CUDA graph"}
    sc = S.reference_scene_10k(seed=1)
    with S.Sim(sc.params, n_max=len(sc.particles), stream=stream.cuda_stream) as sim:
        sim.upload(sc.particles)
        sec = timed_steps(sim, stream, args.extra_steps, 5)
        out["reference_scene_10k"] = {
            "value": len(sc.particles) * args.extra_steps / sec, "unit": UNIT, "particles": len(sc.particles),
            "steps": args.extra_steps, "ms_per_step": 1e3 * sec / args.extra_steps,
            "workload": "10,000 particles, 0.5h lattice in the lower-corner quarter of the reference box"}
    out["render_1m"] = render_workload(stream)
    return out


def render_workload(stream, frames: int = 20) -> dict:
    """The toon draw of the 1M dam break after 200 steps (sph_render into a device buffer,
    1920 x 1080, 4-pixel sprites), timed with CUDA events per frame."""
    import torch
    import nprsph as S

    sc = S.dam_break(seed=2)
    w, h = 1920, 1080
    v = S.view_default(w, h, 1.0)
    S.view_camera(v, 0.0, 1.0, (2.56, 2.5, 6.0), (2.56, 0.5, 0.64))
    v.point_size = 4.0
    img = torch.zeros(w * h * 4, dtype=torch.uint8, device="cuda")
    with S.Sim(sc.params, n_max=len(sc.particles), stream=stream.cuda_stream) as sim:
        sim.upload(sc.particles)
        sim.step(200)
        for _ in range(3):
            sim.render_device(v, img.data_ptr())
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(frames):
            sim.render_device(v, img.data_ptr())
        b.record(stream)
        torch.cuda.synchronize()
    ms = a.elapsed_time(b) / frames
    return {"frames_per_s": 1e3 / ms, "ms_per_frame": ms, "particles": len(sc.particles), "image": [w, h],
            "point_size": 4.0, "frames": frames,
            "workload": "toon draw (splat + depth test + cel shading + Sobel outline) of the 1M dam break at step "
                        "200 into a device RGBA8 buffer"}


WEIGHTS = REPO / "npr-sph_gb300" / "weights" / "mpnn_w64.npy"


def slosh_study(args, stream, total: int = 2000, every: int = 200) -> dict:
    """Learned vs plain on the 16,777,216-particle slosh (256^3 lattice at 0.5h in a 2:1:1 box,
    v_x = 0.5 sin(pi x / L)): `total` dt-equivalents each from the same state (the learned path
    judged every 8 macro-steps: 1% per-particle density deviation, 5% maximum density, 5%
    momentum). Every `every` dt: the FP64 GPU reductions of both runs (momentum, energy, density
    drift from t = 0) and the learned run's density deviation from the plain run by particle id
    (mean and max)."""
    import torch
    import nprsph as S

    if not WEIGHTS.exists():
        return {"unavailable": f"no trained weights at {WEIGHTS.relative_to(REPO)}"}
    params = np.load(WEIGHTS).astype(np.float32)
    sc = S.slosh_block(256, seed=5)
    n = len(sc.particles)

    def diag(sim):
        d = sim.reduce()
        e = d.kinetic_energy + d.potential_energy
        return {"momentum": list(d.momentum), "energy": e, "mean_rho": d.mean_rho, "max_rho": d.max_rho,
                "nonfinite": int(d.nonfinite)}

    rows, reps = [], []
    t_plain = t_learned = 0.0
    with S.Net(16, stream=stream.cuda_stream) as net, \
            S.Sim(sc.params, n_max=n, stream=stream.cuda_stream) as plain, \
            S.Sim(sc.params, n_max=n, stream=stream.cuda_stream) as learned:
        net.set_params(params)
        for sim in (plain, learned):
            sim.upload(sc.particles)
            sim.refresh_density()
        learned.set_max_density_tol(0.05)
        d0p, d0l = diag(plain), diag(learned)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for k in range(total // every):
            torch.cuda.synchronize()
            a.record(stream)
            plain.step(every)
            b.record(stream)
            torch.cuda.synchronize()
            t_plain += a.elapsed_time(b) / 1e3
            a.record(stream)
            reps.append(learned.learned_step(net, every // 4, 8, 0.01, 0.05))
            b.record(stream)
            torch.cuda.synchronize()
            t_learned += a.elapsed_time(b) / 1e3
            plain.refresh_density()
            learned.refresh_density()
            dp, dl = diag(plain), diag(learned)
            rp = plain.download()["extras"][:, 0].astype(np.float64)
            rl = learned.download()["extras"][:, 0].astype(np.float64)
            dev = np.abs(rl - rp) / rp
            m0 = np.linalg.norm(d0p["momentum"]) + 1e-30
            rows.append({
                "dt": (k + 1) * every,
                "learned_vs_plain_density_dev": {"mean": float(dev.mean()), "max": float(dev.max())},
                "plain": {"momentum_drift": float(np.linalg.norm(np.subtract(dp["momentum"], d0p["momentum"])) / m0),
                          "energy_drift": (dp["energy"] - d0p["energy"]) / abs(d0p["energy"]),
                          "mean_rho": dp["mean_rho"], "nonfinite": dp["nonfinite"]},
                "learned": {"momentum_drift": float(np.linalg.norm(np.subtract(dl["momentum"], d0l["momentum"])) / m0),
                            "energy_drift": (dl["energy"] - d0l["energy"]) / abs(d0l["energy"]),
                            "mean_rho": dl["mean_rho"], "nonfinite": dl["nonfinite"]},
            })
    nl = sum(r.learned_macro_steps for r in reps)
    npl = sum(r.plain_macro_steps for r in reps)
    return {"workload": f"slosh 256^3 = 16,777,216 particles, 2:1:1 box, v_x = 0.5 sin(pi x / L), {total} dt-equivalents",
            "particles": n, "plain_updates_per_s": n * total / t_plain, "learned_updates_per_s": n * total / t_learned,
            "learned_macro_steps": nl, "plain_macro_steps": npl, "judged": sum(r.judged for r in reps),
            "fallbacks": sum(r.fallbacks for r in reps), "checkpoints": rows,
            "drift_reference": "FP64 GPU reductions (sph_reduce) of each run against its own t = 0"}


CROP_STEPS = 20


def slosh_crop_fp64(stream) -> dict:
    """The precision study's CPU leg: a 1,048,576-particle crop of the 16.8M slosh (the corner
    column x < 64 s, z < 64 s of the 256^3 lattice, in the slosh's box), 20 dt of plain FP32 GPU
    steps and of learned BF16 macro-steps (unjudged), each against 20 FP64 CPU oracle steps
    from the same state: mean and max per-particle density error, momentum and kinetic-energy
    difference."""
    import nprsph as S
    from oracle import oracle as O

    if not WEIGHTS.exists():
        return {"unavailable": f"no trained weights at {WEIGHTS.relative_to(REPO)}"}
    sc = S.slosh_block(256, seed=5)
    s = 0.5 * sc.params.h
    p = sc.particles
    part = np.ascontiguousarray(p[(p["pos"][:, 0] < 64 * s) & (p["pos"][:, 2] < 64 * s)])
    n = len(part)
    params = sc.params
    pos = np.ascontiguousarray(part["pos"][:, :3], dtype=np.float64)
    vel = np.ascontiguousarray(part["vel"][:, :3], dtype=np.float64)
    t0 = time.perf_counter()
    O.run_f64(params, pos, vel, CROP_STEPS)
    fin = S.empty_particles(n)
    fin["pos"][:, :3] = pos
    fin["pos"][:, 3] = 1.0
    rho64 = O.step_f64(params, fin)["rho"]
    cpu_s = time.perf_counter() - t0
    m = float(np.float32(params.mass))

    def errors(g):
        rho = g["extras"][:, 0].astype(np.float64)
        v = g["vel"][:, :3].astype(np.float64)
        d = np.abs(rho - rho64) / rho64
        return {"density_err_mean": float(d.mean()), "density_err_max": float(d.max()),
                "momentum_diff_rel": float(np.linalg.norm(m * v.sum(0) - m * vel.sum(0)) / (m * np.abs(vel).sum())),
                "kinetic_energy_diff_rel": float(abs((v ** 2).sum() - (vel ** 2).sum()) / (vel ** 2).sum())}

    out = {"particles": n, "dt": CROP_STEPS, "oracle_seconds": cpu_s}
    with S.Sim(params, n_max=n, stream=stream.cuda_stream) as sim, S.Net(16, stream=stream.cuda_stream) as net:
        sim.upload(part)
        sim.step(CROP_STEPS)
        sim.refresh_density()
        out["plain_fp32"] = errors(sim.download())
        for name, w in (("learned_bf16", np.load(WEIGHTS).astype(np.float32)),
                        ("zero_network", np.zeros(int(S.lib.sph_mpnn_num_params()), np.float32))):
            net.set_params(w)
            sim.upload(part)
            sim.learned_step(net, CROP_STEPS // 4, 0)
            sim.refresh_density()
            out[name] = errors(sim.download())
    return out


def learned_workload(args, stream, flush) -> dict:
    """The learned macro-step on the same dam break: units of 8 macro-steps (32 dt, the last one
    judged against 4 plain steps from the same state), each timed with CUDA events, L2 flushed
    between units; plain SPH timed the same way over the same interval; the end states compared.
    Run once per judge metric: the deviation of the mean density (the default) and the mean
    per-particle density deviation."""
    import torch
    import nprsph as S

    if not WEIGHTS.exists():
        return {"unavailable": f"no trained weights at {WEIGHTS.relative_to(REPO)}"}
    params = np.load(WEIGHTS).astype(np.float32)
    sc = S.dam_break(seed=2)
    n = len(sc.particles)
    units = max(1, args.steps // 32)
    judge_every, tol, mtol, xtol = 8, 0.01, 0.05, 0.05

    def timed_units(fn) -> float:
        total = 0.0
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for _ in range(units):
            with torch.cuda.stream(stream):
                flush.add_(1.0)
            torch.cuda.synchronize()
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            total += a.elapsed_time(b) / 1e3
        return total

    def summary(reps, t_l, t_p, rl, rp) -> dict:
        judged = sum(r.judged for r in reps)
        n_learned = sum(r.learned_macro_steps for r in reps)
        n_plain = sum(r.plain_macro_steps for r in reps)
        return {
            "value": n * 32 * units / t_l, "unit": UNIT, "ms_per_dt": 1e3 * t_l / (32 * units),
            "speedup_vs_plain": t_p / t_l, "judged": judged, "fallbacks": sum(r.fallbacks for r in reps),
            "learned_macro_steps": n_learned, "plain_macro_steps": n_plain,
            "discarded_macro_steps": sum(r.discarded_macro_steps for r in reps),
            "learned_fraction": n_learned / max(n_learned + n_plain, 1),
            "judged_mean_rho_dev_max": max((r.max_mean_rho_dev for r in reps), default=0.0),
            "judged_max_rho_dev_max": max((r.max_max_rho_dev for r in reps), default=0.0),
            "judged_particle_density_dev_mean": sum(r.sum_density_dev for r in reps) / max(judged, 1),
            "judged_particle_density_dev_max": max((r.max_density_dev for r in reps), default=0.0),
            "end_state_vs_plain_run": {
                "mean_rho_dev": float(abs(rl.sum() - rp.sum()) / rp.sum()),
                "particle_density_dev_mean": float(np.mean(np.abs(rl - rp) / rp)),
                "particle_density_dev_max": float(np.max(np.abs(rl - rp) / rp))},
        }

    out = {"workload": "dam break 1,048,576 particles (as above), learned macro-steps of 4 dt in intervals of 8; "
                       "the last macro-step of each interval is judged against 4 plain steps from the same state "
                       "(tolerance 1% density deviation, 5% deviation of the maximum density, 5% momentum difference "
                       "relative to sum m|v| + M|G|4dt); a failed interval is rolled back and run by plain SPH. "
                       "Density deviation of the judge: the mean over particles of |rho_learned - rho_plain| / "
                       "rho_plain (the default), and, in 'judge_mean_density', the deviation of the mean density "
                       "|sum rho_learned - sum rho_plain| / sum rho_plain (FP64 reductions)",
           "units": units, "macro_steps": units * judge_every, "dt_equivalents": units * 32}
    runs = {}
    with S.Net(16, stream=stream.cuda_stream) as net, \
            S.Sim(sc.params, n_max=n, stream=stream.cuda_stream) as learned, \
            S.Sim(sc.params, n_max=n, stream=stream.cuda_stream) as plain:
        net.set_params(params)
        plain.upload(sc.particles)
        plain.step(args.warmup + 32)
        t_p = timed_units(lambda: plain.step(32))
        plain.refresh_density()
        b = plain.download()
        rp = b["extras"][:, 0].astype(np.float64)
        for name, metric in (("judge_particle_density", S.JUDGE_PARTICLE_DENSITY),
                             ("judge_mean_density", S.JUDGE_MEAN_DENSITY)):
            reps = []
            learned.upload(sc.particles)
            learned.set_judge(metric)
            learned.set_max_density_tol(xtol)
            learned.step(args.warmup)
            learned.learned_step(net, judge_every, judge_every, tol, mtol)  # warm-up unit (allocations)
            t_l = timed_units(lambda: reps.append(learned.learned_step(net, judge_every, judge_every, tol, mtol)))
            learned.refresh_density()
            rl = learned.download()["extras"][:, 0].astype(np.float64)
            runs[name] = summary(reps, t_l, t_p, rl, rp)
        learned.set_judge(S.JUDGE_PARTICLE_DENSITY)
        learned.set_max_density_tol(float("inf"))
        # One unjudged macro-step (sort, neighbour lists, two inference rounds, update) with each
        # BF16 inference kernel set, from the same state, CUDA events over 8 macro-steps.
        kernels = {}
        for name, prec in (("tcgen05_round1_lanes+mma_sync_round2 (default)", 3), ("mma_sync", 1),
                           ("tcgen05_edges_on_lanes", 2)):
            net.set_precision(prec)
            learned.upload(sc.particles)
            learned.step(args.warmup)
            learned.learned_step(net, 2, 0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            learned.learned_step(net, 8, 0)
            e1.record(stream)
            torch.cuda.synchronize()
            kernels[name] = {"ms_per_macro_step": e0.elapsed_time(e1) / 8}
        net.set_precision(3)
        # BF16 tensor-core bound of the learned macro-step: its algorithmic flops from the layer
        # shapes (fixed 32 neighbour slots, padded ones included), per particle and macro-step,
        # over the default kernel set's CUDA-event time, against the sustained cuBLAS BF16 rate.
        K_NB, W_H, F_E, F_N, F_O = 32, 64, 14, 9, 6
        flop = 2 * (2 * K_NB * F_E * W_H) + 2 * ((W_H + F_N) * W_H + W_H * W_H) + 2 * (2 * W_H * W_H + W_H * F_O)
        peaks, psrc = measured_peaks()
        peak = float(peaks.get("bf16_tflops_sustained", peaks["bf16_tflops"]))
        ms_macro = kernels["tcgen05_round1_lanes+mma_sync_round2 (default)"]["ms_per_macro_step"]
        achieved = flop * n / (ms_macro * 1e-3) / 1e12
        tensor_roofline = {
            "bound": "tensor", "flop_per_particle_per_macro_step": flop,
            "flop_model": "2 rounds x 32 edges x 14 x 64 edge MACs, node layers 73x64 + 64x64 (round 1), "
                          "128x64 + 64x6 (round 2 and output); 2 flop per MAC",
            "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "peak_source": f"{psrc} bf16_tflops_sustained" if "bf16_tflops_sustained" in peaks else f"{psrc} bf16_tflops",
            "ms_per_macro_step": ms_macro,
        }
        # What the network gains: one judged macro-step from the same state (the plain run's
        # end state) with the trained network and with a zero network (v' = v, x' = x + 4 dt v,
        # then the momentum projection adds gravity).
        gain = {}
        with S.Net(16, stream=stream.cuda_stream) as zero:
            zero.set_params(np.zeros(int(S.lib.sph_mpnn_num_params()), np.float32))
            for name, nn in (("trained", net), ("zero_network", zero)):
                learned.upload(b)
                r = learned.learned_step(nn, 1, 1, 1e30, 1e30)
                gain[name] = {"mean_rho_dev": r.last_mean_rho_dev, "max_rho_dev": r.last_max_rho_dev,
                              "particle_density_dev": r.last_density_dev, "momentum_dev": r.last_momentum_dev}
    out.update(runs["judge_particle_density"])
    out.update({
        "plain_value": n * 32 * units / t_p, "plain_ms_per_dt": 1e3 * t_p / (32 * units),
        "judge_mean_density": runs["judge_mean_density"],
        "one_macro_step_vs_4_plain_steps": gain,
        "inference_kernels": kernels,
        "tensor_roofline": tensor_roofline,
        "precision": "BF16 weights/activations, FP32 accumulate: round 1 tcgen05 MMAs (TMEM accumulators), "
                     "round 2 mma.sync m16n8k16; every kernel set is timed in inference_kernels",
        "weights": str(WEIGHTS.relative_to(REPO)),
    })
    return out


FP32_LANES_PER_SM = 128  # FP32 FMA lanes per SM (4 sub-partitions x 32)
# FP32 work per unit: a candidate test (3 sub, 3 mul/FMA, the compare: ~9 flop),
# a density interaction (~10), a force interaction (~40).
FLOP_CAND, FLOP_DENS, FLOP_FORCE = 9, 10, 40


def roofline_block(n, steps, pass_avg, step_s, cand, pairs, hbm, src, peaks, dev) -> dict:
    """HBM and FP32-pipe rooflines of the dominant pair kernel and of the whole step. Bytes:
    the algorithmic bytes per particle of each pass over its CUDA-event time. Flops: the
    on-device counters of this run's trajectory times the per-unit flops, over the same
    time; peak FP32 = SMs x 128 lanes x 2 flop x the maximum SM clock."""
    import torch

    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    mhz = float(peaks.get("sm_max_mhz", 2070.0))
    fp32_peak = sms * FP32_LANES_PER_SM * 2 * mhz * 1e6 / 1e12  # TFLOP/s
    flops = {"density": (FLOP_CAND * cand + FLOP_DENS * pairs) / steps,
             "force_integrate": FLOP_FORCE * (pairs - n * steps) / steps}
    per = {}
    for k, ms in (("density", pass_avg[1]), ("force_integrate", pass_avg[2])):
        gbs = B_ALG[k] * n / (ms * 1e-3) / 1e9
        tfl = flops[k] / (ms * 1e-3) / 1e12
        per[k] = {"ms": ms, "hbm_achieved": gbs, "hbm_frac": gbs / hbm, "fp32_achieved": tfl,
                  "fp32_frac": tfl / fp32_peak, "bytes_per_particle": B_ALG[k], "flop_per_particle": flops[k] / n}
    kern = max(per, key=lambda k: per[k]["ms"])
    d = per[kern]
    bound = "fp32" if d["fp32_frac"] > d["hbm_frac"] else "hbm"
    step_gbs = B_ALG_STEP * n * steps / step_s / 1e9
    step_tfl = (flops["density"] + flops["force_integrate"]) * steps / step_s / 1e12
    traffic = profiled_traffic("k_" + kern)
    return {
        "bound": bound, "kernel": kern,
        "achieved": d["fp32_achieved"] if bound == "fp32" else d["hbm_achieved"],
        "peak": fp32_peak if bound == "fp32" else hbm,
        "unit": "TFLOP/s" if bound == "fp32" else "GB/s",
        "frac": d["fp32_frac"] if bound == "fp32" else d["hbm_frac"],
        "traffic": traffic,
        "traffic_source": f"ncu dram__bytes_read.sum + dram__bytes_write.sum of one k_{kern} launch at the "
                          f"dense start, cold L2, from the capture summarised in {PROFILE} (not measured in this run)",
        "hbm_peak": hbm, "hbm_peak_source": f"{src} hbm_gbs",
        "fp32_peak": fp32_peak, "fp32_peak_source": f"{sms} SMs x {FP32_LANES_PER_SM} lanes x 2 flop x {mhz:.0f} MHz",
        "passes": per,
        "work_counters": {"candidate_tests_per_particle": cand / (n * steps),
                          "pairs_per_particle_incl_self": pairs / (n * steps),
                          "flop_model": f"{FLOP_CAND} per candidate test, {FLOP_DENS} per density and "
                                        f"{FLOP_FORCE} per force interaction"},
        "step_achieved": step_gbs, "step_frac": step_gbs / hbm, "step_bytes_per_particle": B_ALG_STEP,
        "step_fp32_achieved": step_tfl, "step_fp32_frac": step_tfl / fp32_peak,
    }


def run_ours(args) -> None:
    import torch
    import nprsph as S

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.Stream(device=dev)
    sc = S.dam_break(seed=2 + rank)
    n = len(sc.particles)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    sim = S.Sim(sc.params, n_max=n, stream=stream.cuda_stream)
    if args.autotune:
        sim.upload(sc.particles)
        sim.autotune(5)
    sim.upload(sc.particles)
    sim.step(args.warmup)
    sim.synchronize()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    rec0 = sim.record_stats()
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(dev.index) as clk:
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.add_(1.0)  # L2 flush, outside the timed events
                ev[k][0].record(stream)
                sim.step(1)
                ev[k][1].record(stream)
        torch.cuda.synchronize()
    sim.synchronize()
    barrier(world)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    local_s = sum(step_ms) / 1e3
    total_s = max_over_ranks(local_s, world)
    diag = sim.reduce()
    fallback = sim.tile_stats()
    rec1 = sim.record_stats()

    # Per-pass device times over the same trajectory (events between passes, eager launches).
    sim.upload(sc.particles)
    sim.step(args.warmup)
    sim.enable_timing(True)
    with torch.cuda.stream(stream):
        pass_ms = np.zeros(3)
        for k in range(args.steps):
            flush.add_(1.0)
            sim.step(1)
            pass_ms += np.array(sim.pass_times())
    sim.enable_timing(False)
    pass_avg = pass_ms / args.steps

    # Work of the pair passes over the same trajectory, from on-device counters: candidate
    # tests and r < h pairs of each step's density pass (the force pass interacts with the
    # pairs other than the particle itself).
    sim.upload(sc.particles)
    sim.step(args.warmup)
    cand = pairs = 0
    for k in range(args.steps):
        c, pr = sim.pair_counts()
        cand += c
        pairs += pr
        sim.step(1)
    sim.synchronize()

    # End to end through the C ABI with host buffers: upload + step + download each step.
    host_in = torch.empty(n * 64, dtype=torch.uint8, pin_memory=True).numpy().view(S.PARTICLE_DTYPE)
    host_out = torch.empty(n * 64, dtype=torch.uint8, pin_memory=True).numpy().view(S.PARTICLE_DTYPE)
    host_in[:] = sc.particles
    sim.upload(host_in)
    sim.step(args.warmup)
    sim.download(host_in)
    e2e_steps = min(args.steps, 200)
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        sim.upload(host_in)
        sim.step(1)
        sim.download(host_out)
        host_in, host_out = host_out, host_in
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    blk, sten = sim.get_launch()
    sim.close()

    if rank != 0:
        return
    extra = extra_workloads(args, stream) if args.extra_steps > 0 else {}
    learned = learned_workload(args, stream, flush) if args.learned else {"skipped": "--no-learned"}
    if args.learned:
        # config 5: the full study (2,000 dt) with --study, else a short leg of 200 dt
        learned["slosh_16m_study"] = slosh_study(args, stream, 2000, 200) if args.study else \
            slosh_study(args, stream, 200, 100)
        learned["slosh_16m_study"]["crop_1m_vs_fp64_oracle"] = slosh_crop_fp64(stream)
    peaks, src = measured_peaks()
    hbm = float(peaks["hbm_gbs"])
    value = world * n * args.steps / total_s
    clocks = clk.summary()
    roofline = roofline_block(n, args.steps, pass_avg, local_s, cand, pairs, hbm, src, peaks, dev)
    cpu = cpu_oracle_legs(args.warmup, min(args.steps, args.cpu_steps)) if args.cpu_steps > 0 else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps,
        "ms_per_step_by_tenth": [round(float(np.mean(w)), 4) for w in np.array_split(np.array(step_ms), 10) if len(w)],
        "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD,
                   "particles": n, "timed_steps": [args.warmup, args.warmup + args.steps],
                   "l2": "flushed between steps (256 MiB write outside the timed events)",
                   "launch": {"threads_per_block": blk, "stencil": sten}, "parallelism": f"replicas x{world}",
                   "global_path_chunks": {"density": fallback[0], "force": fallback[1],
                                          "of": (args.warmup + args.steps) * ((n + blk - 1) // blk)},
                   "neighbour_records": {"timed_steps_with": rec1[0] - rec0[0],
                                         "timed_steps_without": rec1[1] - rec0[1]}},
        "roofline": roofline,
        "passes_ms": {"sort": pass_avg[0], "density": pass_avg[1], "force_integrate": pass_avg[2]},
        "cpu_baseline": cpu,
        "e2e": {"value": world * n * e2e_steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": n * 64,
                "d2h_bytes_per_step": n * 64, "steps": e2e_steps,
                "path": "sph_upload_aos + sph_step(1) + sph_download_aos, pinned host AoS records"},
        "gpu_launches": KERNELS_PER_STEP * args.steps,
        "clocks": clocks,
        "final_state": {"mean_rho": diag.mean_rho, "nonfinite": int(diag.nonfinite), "step": int(diag.step)},
        "other_configs": extra,
        "learned": learned,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-steps", type=int, default=CPU_STEPS_MAX,
                    help="cap on the timed steps of the CPU oracle leg (0: skip it)")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="keep the default launch shape instead of timing the candidates first")
    ap.add_argument("--no-learned", dest="learned", action="store_false",
                    help="skip the learned macro-step measurement")
    ap.add_argument("--study", action="store_true",
                    help="run the 16M-particle slosh study of learned vs plain over 2,000 dt-equivalents "
                         "(default: 200)")
    ap.add_argument("--extra-steps", type=int, default=100,
                    help="steps of the batched-scenes and 10k reference-scene measurements (0: skip)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
