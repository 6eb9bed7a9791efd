"""Precision study on a 1,048,576-particle crop of the 16,777,216-particle slosh (the corner
column x < 64 s, z < 64 s of the 256^3 lattice, in the slosh's 2:1:1 box): 20 dt of plain FP32
GPU steps and of BF16 learned macro-steps (trained, and a zero network for comparison), each
against 20 FP64 CPU oracle steps from the same state. Reports mean/max density error, momentum and energy drift; writes them as JSON to
$SPH_STUDY_OUT when that is set."""
from __future__ import annotations

import json
import os
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WEIGHTS = Path(__file__).resolve().parents[1] / "npr-sph_gb300" / "weights" / "mpnn_w64.npy"
# Bounds on the crop after 20 dt against the FP64 oracle. Plain FP32: 1e-3 (measured ~1e-6).
# Learned BF16 (5 unjudged macro-steps): mean per-particle density error 10% (measured 6.5%;
# the network misses the 1% of a judged interval here, which is why the judge exists), and the
# trained network must beat the macro-step without it on every measure.
PLAIN_TOL = 1e-3
LEARNED_DENSITY_TOL = 0.10


def crop(sph):
    sc = sph.slosh_block(256, seed=5)
    s = 0.5 * sc.params.h
    p = sc.particles
    keep = (p["pos"][:, 0] < 64 * s) & (p["pos"][:, 2] < 64 * s)
    part = np.ascontiguousarray(p[keep])
    assert len(part) == 64 * 256 * 64
    return sc.params, part


def errors(rho, rho64, vel, vel64, m):
    d = np.abs(rho - rho64) / rho64
    p32, p64 = m * vel.sum(0), m * vel64.sum(0)
    e32, e64 = 0.5 * m * (vel ** 2).sum(), 0.5 * m * (vel64 ** 2).sum()
    return {"density_err_mean": float(d.mean()), "density_err_max": float(d.max()),
            "momentum_diff_rel": float(np.linalg.norm(p32 - p64) / (m * np.abs(vel64).sum())),
            "kinetic_energy_diff_rel": float(abs(e32 - e64) / e64)}


def test_crop_fp32_and_learned_against_fp64(sph, orc, gpu):
    params, part = crop(sph)
    n = len(part)
    steps = 20
    pos = np.ascontiguousarray(part["pos"][:, :3], dtype=np.float64)
    vel = np.ascontiguousarray(part["vel"][:, :3], dtype=np.float64)
    rho64, _ = orc.run_f64(params, pos, vel, steps)  # in place: pos, vel after `steps` steps
    # the oracle's rho is of the last step's density pass; the comparison needs rho at the
    # final positions: one more density evaluation
    fin = sph.empty_particles(n)
    fin["pos"][:, :3] = pos
    fin["pos"][:, 3] = 1.0
    rho64 = orc.step_f64(params, fin)["rho"]
    out = {"particles": n, "steps": steps}
    with sph.Sim(params, n_max=n) as sim:
        sim.upload(part)
        sim.step(steps)
        sim.refresh_density()
        g = sim.download()
        out["plain_fp32"] = errors(g["extras"][:, 0].astype(np.float64), rho64, g["vel"][:, :3].astype(np.float64),
                                   vel, params.mass)
        if WEIGHTS.exists():
            from oracle import mpnn_oracle as MO

            for name, w in (("learned_bf16", np.load(WEIGHTS).astype(np.float32)),
                            ("zero_network", np.zeros(MO.n_params(), np.float32))):
                with sph.Net(16) as net:
                    net.set_params(w)
                    sim.upload(part)
                    rep = sim.learned_step(net, steps // 4, 0)
                    assert rep.learned_macro_steps == steps // 4
                    sim.refresh_density()
                    g = sim.download()
                out[name] = errors(g["extras"][:, 0].astype(np.float64), rho64, g["vel"][:, :3].astype(np.float64),
                                   vel, params.mass)
    if os.environ.get("SPH_STUDY_OUT"):
        Path(os.environ["SPH_STUDY_OUT"]).write_text(json.dumps(out, indent=1))
    print(json.dumps(out))
    assert out["plain_fp32"]["density_err_mean"] < PLAIN_TOL
    assert out["plain_fp32"]["momentum_diff_rel"] < PLAIN_TOL
    if "learned_bf16" in out:  # the trained network beats the macro-step without it (v' = v, x' = x + 4 dt v)
        assert out["learned_bf16"]["density_err_mean"] < LEARNED_DENSITY_TOL
        for k in ("density_err_mean", "momentum_diff_rel", "kinetic_energy_diff_rel"):
            assert out["learned_bf16"][k] < out["zero_network"][k], k
