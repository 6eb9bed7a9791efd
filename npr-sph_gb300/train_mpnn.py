"""Train the learned macro-step network on trajectories the GPU SPH step generates.

    python npr-sph_gb300/train_mpnn.py [--scenes 200] [--particles 65536] [--frames 24]
                                       [--gap 8] [--steps 60000] [--rollout-schedule 8:7:60000,...]
                                       [--out npr-sph_gb300/weights/mpnn_w64.npy]

Training data: `scenes` seeded runs of `particles` particles each, advanced together in one
batched context with the literal mass and smoothing length and g = -9.81. Per run the stiffness k
and viscosity mu and the drop geometry are drawn from the seed:
  - even runs: a dam break, a block against the x = 0 wall of a 4:1:1 box, k ~ U[1500, 2500],
    mu = 3000 * U[0.5, 1.5] (around the literal uniforms);
  - odd runs: a lattice block in the lower corner, or a ball dropped from mid-height, of a cubic
    box, k ~ U[500, 3000], mu log-uniform in [0.1, 3000].
Every `gap` steps each run contributes a frame: its state, the <= 32 nearest neighbours and
density of every particle, and as targets the mean accelerations of the next 4 plain steps
(the velocity head O_v and the position head O_x, in units of k/h) from the forces. The network is then trained by Adam on the GPU (the library's own forward and
backward kernels), one frame per step, with a cosine-decayed learning rate. By default the
node layers and all weight gradients run as BF16 GEMMs on the tensor cores (FP32 accumulation,
FP32 master weights); --precision 0 runs every layer in FP32.

Rollout rounds (--rollout-schedule) then fine-tune the network on states it produces itself:
a macro-step judged after a run of learned macro-steps starts from such a state, and a network
trained on plain-SPH states alone errs more there. Each round re-records the plain frames and,
per run, `frames` rollouts: the run's initial state, plain SPH for 8-192 steps, 1-`macro`
unjudged learned macro-steps of the current network (BF16 inference), and a frame recorded
there, its targets again from 4 plain steps. Adam then runs `steps` steps over both kinds of
frames from the current weights, the learning rate cosine-decayed from --rollout-lr.
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

import nprsph as S  # noqa: E402

DEFAULT_OUT = HERE / "weights" / "mpnn_w64.npy"


def training_scenes(n_scene: int, n: int, seed: int):
    rng = np.random.default_rng(seed)
    p0 = S.default_params()
    s = 0.5 * p0.h
    plist, parts = [], []
    for i in range(n_scene):
        if i % 2 == 0:
            nx = int(round(n ** (1 / 3) / 2 ** (1 / 3)))   # block nx x 2nx x nx ~ n
            while nx * 2 * nx * nx < n:
                nx += 1
            by, bz = 2 * nx * s, nx * s
            L = max(by, bz)
            p = S.workload_params(lower=(0.0, 0.0, 0.0), upper=(4 * L, by, bz),
                                  k=float(rng.uniform(1500, 2500)), mu=float(3000.0 * rng.uniform(0.5, 1.5)),
                                  flags=S.FLAG_KEEP_FORCE)
            a = S.scene_fill(n, (0.0, 0.0, 0.0), (nx * s, by, bz), s, 0.01 * p.h, seed * 7919 + i)
        else:
            edge = 2.0 * math.ceil(n ** (1 / 3) + 1) * s
            p = S.workload_params(lower=(0.0, 0.0, 0.0), upper=(edge, edge, edge), k=float(rng.uniform(500, 3000)),
                                  mu=float(10 ** rng.uniform(-1, math.log10(3000.0))), flags=S.FLAG_KEEP_FORCE)
            if rng.integers(0, 2):
                a = S.scene_ball(n, (0.5 * edge, 0.55 * edge, 0.5 * edge), s, 0.01 * p.h, seed * 7919 + i)
            else:
                a = S.scene_fill(n, (0.0, 0.0, 0.0), (0.5 * edge, edge, 0.5 * edge), s, 0.01 * p.h, seed * 7919 + i)
        plist.append(p)
        parts.append(a)
    counts = np.full(n_scene, n, dtype=np.uint32)
    return plist, counts, np.concatenate(parts)


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--scenes", type=int, default=200)
    ap.add_argument("--particles", type=int, default=65536)
    ap.add_argument("--frames", type=int, default=24, help="frames per run")
    ap.add_argument("--gap", type=int, default=8, help="plain steps between frames")
    ap.add_argument("--steps", type=int, default=60000, help="Adam steps")
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=4)
    ap.add_argument("--precision", type=int, default=1, choices=[0, 1],
                    help="1: node layers and weight gradients as BF16 tensor-core (tcgen05) GEMMs; 0: FP32")
    ap.add_argument("--rollout-schedule", default="8:7:60000,16:8:60000,16:8:60000,24:24:120000",
                    help="rollout rounds frames:macro:steps, comma-separated ('' for none)")
    ap.add_argument("--rollout-lr", type=float, default=3e-4)
    ap.add_argument("--rollout-plain-max", type=int, default=192,
                    help="a rollout starts after 8 .. this many plain steps (a multiple of 8)")
    ap.add_argument("--init", type=Path, default=None,
                    help="start from these parameters (with --steps 0: rollout rounds only)")
    ap.add_argument("--out", type=Path, default=DEFAULT_OUT)
    args = ap.parse_args()

    t0 = time.time()
    plist, counts, parts = training_scenes(args.scenes, args.particles, args.seed)
    net = S.Net(args.particles)
    net.set_params(np.load(args.init).astype(np.float32) if args.init else init_params(args.seed))
    net.set_train_precision(args.precision)
    with S.Sim(plist, counts=counts) as sim:
        sim.upload(parts)
        for f in range(args.frames):
            total = net.record(sim, 1)
            if f + 1 < args.frames:
                sim.step(args.gap)
        sim.synchronize()
    t_rec = time.time() - t0
    t1 = time.time()
    loss = train_steps(net, args.steps, args.lr, args.seed * 1000003) if args.steps > 0 else np.zeros(0)
    t_train = time.time() - t1
    rounds = []
    for r, spec in enumerate(x for x in args.rollout_schedule.split(",") if x):
        frames, macro, steps = (int(v) for v in spec.split(":"))
        t2 = time.time()
        net.clear_frames()
        with S.Sim(plist, counts=counts) as sim:
            sim.upload(parts)
            for f in range(args.frames):
                n_plain = net.record(sim, 1)
                if f + 1 < args.frames:
                    sim.step(args.gap)
            sim.synchronize()
        n_roll = rollout_frames(net, plist, counts, parts, frames, macro, args.seed + 99 + r,
                                plain_max=args.rollout_plain_max)
        t3 = time.time()
        rl = train_steps(net, steps, args.rollout_lr, args.seed * 1000003 + 77 + 1000 * r)
        rounds.append({"rollout_frames_per_run": frames, "max_macro_steps": macro, "adam_steps": steps,
                       "frames": {"plain": int(n_plain), "rollout": int(n_roll - n_plain)},
                       "loss_first_500": float(rl[:500].mean()), "loss_last_500": float(rl[-500:].mean()),
                       "record_s": t3 - t2, "train_s": time.time() - t3})
        print(json.dumps({"rollout_round": r, **rounds[-1]}), flush=True)
    params = net.get_params()
    net.close()
    args.out.parent.mkdir(parents=True, exist_ok=True)
    np.save(args.out, params)
    meta = {"scenes": args.scenes, "particles": args.particles, "frames_per_run": args.frames, "gap": args.gap,
            "frames": int(total), "adam_steps": args.steps, "lr": args.lr, "seed": args.seed,
            "train_precision": "bf16 tcgen05 GEMMs" if args.precision == 1 else "fp32",
            "loss_first_500": float(loss[:500].mean()) if len(loss) else None,
            "loss_last_500": float(loss[-500:].mean()) if len(loss) else None,
            "record_s": t_rec, "train_s": t_train, "init": str(args.init) if args.init else None,
            "rollout_lr": args.rollout_lr, "rollout_plain_max": args.rollout_plain_max, "rollout_rounds": rounds}
    args.out.with_suffix(".json").write_text(json.dumps(meta, indent=1))
    print(json.dumps(meta))


def train_steps(net, steps: int, lr0: float, seed: int) -> np.ndarray:
    """`steps` Adam steps over the recorded frames, the learning rate cosine-decayed from lr0 to lr0/100."""
    losses, done, chunk = [], 0, 500
    while done < steps:
        k = min(chunk, steps - done)
        lr = lr0 * (0.01 + 0.99 * 0.5 * (1 + math.cos(math.pi * done / steps)))
        losses.append(net.train(k, lr=lr, seed=seed + done))
        done += k
    return np.concatenate(losses)


def rollout_frames(net, plist, counts, parts, per_run: int, macro: int, seed: int, plain_max: int = 192) -> int:
    """Record per_run frames of every run at states the network reached itself: from the run's
    initial state, 8-plain_max plain steps (multiples of 8), then 1-macro unjudged learned
    macro-steps. Returns the frames recorded in total."""
    rng = np.random.default_rng(seed)
    offs = [0] + [int(x) for x in np.cumsum(counts)]
    total = 0
    for i, p in enumerate(plist):
        with S.Sim(p, n_max=int(counts[i])) as sim:
            for _ in range(per_run):
                sim.upload(parts[offs[i]:offs[i + 1]])
                sim.step(int(8 * rng.integers(1, plain_max // 8 + 1)))
                sim.learned_step(net, int(rng.integers(1, macro + 1)), 0, 1e30, 1e30)
                total = net.record(sim, 1)
            sim.synchronize()
    return total


def init_params(seed: int) -> np.ndarray:
    """He-style initial parameters in the library's flat layout (sph_mpnn_set_params)."""
    rng = np.random.default_rng(seed)
    W, FE, FN, FO = 64, 14, 9, 6
    shapes = [("We1", (FE, W)), ("be1", (W,)), ("Wn1", (W + FN, W)), ("bn1", (W,)), ("Wp", (W, W)),
              ("We2", (FE, W)), ("be2", (W,)), ("Wn2", (2 * W, W)), ("bn2", (W,)), ("Wo", (W, FO)), ("bo", (FO,))]
    out = []
    for name, shape in shapes:
        if name.startswith("W"):
            scale = math.sqrt(2.0 / shape[0]) if name != "Wo" else 0.1 / math.sqrt(shape[0])
            out.append(rng.normal(0.0, scale, shape).reshape(-1))
        else:
            out.append(np.zeros(int(np.prod(shape))))
    flat = np.concatenate(out).astype(np.float32)
    assert len(flat) == int(S.lib.sph_mpnn_num_params())
    return flat


if __name__ == "__main__":
    main()
