"""The learned macro-step: GPU forward/backward against the FP64 restatement
(oracle/mpnn_oracle.py), training on frames recorded from the plain step, the judge, and
the gain of the trained network over the same macro-step without it (a zero network:
v' = v, x' = x + 4 dt v), and the judge's roll-back to plain SPH."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def random_frame(seed: int, n: int = 96):
    from oracle import mpnn_oracle as MO

    rng = np.random.default_rng(seed)
    h, c = 0.02, 44.72
    pos = rng.uniform(0.0, 0.06, (n, 3))
    d = np.linalg.norm(pos[:, None, :] - pos[None, :, :], axis=-1)
    nb = np.full((n, MO.K), -1, dtype=np.int32)
    cnt = np.zeros(n, dtype=np.int32)
    for i in range(n):
        js = [j for j in np.argsort(d[i]) if j != i and d[i, j] < h][:MO.K]
        cnt[i] = len(js)
        nb[i, :len(js)] = js
    vel = rng.normal(0.0, 1.0, (n, 3))
    rho = rng.uniform(3900.0, 20000.0, n)
    target = rng.normal(0.0, 0.05, (n, MO.FO))
    dt = 1e-4
    fc = np.array([h, c, 3916.7, 1000.0, np.log10(3000.0) / 4.0, c * dt / h])
    return pos, vel, rho, nb, cnt, target, fc


def frame_dt(fc) -> float:
    """dt with c dt / h equal to the frame's Courant number as the GPU receives it (FP32)."""
    f = np.asarray(fc, np.float32).astype(np.float64)
    return f[5] * f[0] / f[1]


def test_forward_and_gradient_match_fp64_oracle(sph, gpu):
    from oracle import mpnn_oracle as MO

    pos, vel, rho, nb, cnt, target, fc = random_frame(3)
    n = len(pos)
    assert cnt.min() >= 0 and cnt.max() > 4
    f32 = lambda a: np.asarray(a, np.float32).astype(np.float64)  # the GPU sees FP32 inputs
    flat = MO.init_params(7)
    pos4 = np.zeros((n, 4), np.float32); pos4[:, :3] = pos
    vel4 = np.zeros((n, 4), np.float32); vel4[:, :3] = vel
    rhop = np.zeros((n, 2), np.float32); rhop[:, 0] = rho
    tg8 = np.zeros((n, 8), np.float32); tg8[:, :MO.FO] = target
    with sph.Net(128) as net:
        net.set_params(flat)
        net.set_train_precision(0)  # every layer in FP32 on the CUDA cores
        loss, out, grad = net.loss_grad(pos4, vel4, rhop, nb, cnt, tg8, fc)
    e, mask, nf = MO.features(f32(pos), f32(vel), f32(rho), nb, cnt, *[float(np.float32(x)) for x in fc[:2]],
                              float(np.float32(fc[2])), float(np.float32(fc[3])), 3000.0, frame_dt(fc))
    ref_loss, ref_out, ref_grad = MO.loss_and_grad(flat.astype(np.float64), e, mask, nf, nb, f32(target))
    np.testing.assert_allclose(out[:, :MO.FO], ref_out, rtol=0, atol=2e-5 * np.abs(ref_out).max())
    assert np.all(out[:, MO.FO:] == 0.0)
    assert loss == pytest.approx(ref_loss, rel=1e-4)
    off = 0
    for name, shape in MO.LAYOUT:
        size = int(np.prod(shape))
        g, r = grad[off:off + size], ref_grad[off:off + size]
        scale = np.abs(r).max() + 1e-12
        assert np.max(np.abs(g - r)) <= 2e-4 * scale, (name, np.max(np.abs(g - r)) / scale)
        off += size


# BF16 tolerances of the tensor-core training path against the FP64 restatement: the node
# layers round their operands (activations, gradients, weights) to 8 mantissa bits before the
# FP32-accumulated GEMMs, so outputs and gradients agree to a few percent of their scale.
TC_OUT_TOL, TC_GRAD_TOL, TC_LOSS_RTOL, TC_GRAD_CORR = 3e-2, 6e-2, 3e-2, 0.995


@pytest.mark.parametrize("seed", [3, 8])
def test_tensor_core_training_matches_fp64_oracle(sph, gpu, seed):
    """The training passes with the node layers on the BF16 tcgen05 GEMMs (the default training
    precision): outputs, loss and every layer's gradient against the FP64 restatement."""
    from oracle import mpnn_oracle as MO

    pos, vel, rho, nb, cnt, target, fc = random_frame(seed, n=300)
    n = len(pos)
    f32 = lambda a: np.asarray(a, np.float32).astype(np.float64)
    flat = MO.init_params(seed + 4)
    pos4 = np.zeros((n, 4), np.float32); pos4[:, :3] = pos
    vel4 = np.zeros((n, 4), np.float32); vel4[:, :3] = vel
    rhop = np.zeros((n, 2), np.float32); rhop[:, 0] = rho
    tg8 = np.zeros((n, 8), np.float32); tg8[:, :MO.FO] = target
    with sph.Net(512) as net:
        net.set_params(flat)
        loss, out, grad = net.loss_grad(pos4, vel4, rhop, nb, cnt, tg8, fc)
        fwd = net.forward(pos4, vel4, rhop, nb, cnt, fc, precision=2)
    np.testing.assert_array_equal(fwd, out)  # the same forward pass
    e, mask, nf = MO.features(f32(pos), f32(vel), f32(rho), nb, cnt, *[float(np.float32(x)) for x in fc[:2]],
                              float(np.float32(fc[2])), float(np.float32(fc[3])), 3000.0, frame_dt(fc))
    ref_loss, ref_out, ref_grad = MO.loss_and_grad(flat.astype(np.float64), e, mask, nf, nb, f32(target))
    assert np.abs(out[:, :MO.FO] - ref_out).max() <= TC_OUT_TOL * np.abs(ref_out).max()
    assert np.all(out[:, MO.FO:] == 0.0)
    assert loss == pytest.approx(ref_loss, rel=TC_LOSS_RTOL)
    off = 0
    for name, shape in MO.LAYOUT:
        size = int(np.prod(shape))
        g, r = grad[off:off + size].astype(np.float64), ref_grad[off:off + size]
        scale = np.abs(r).max() + 1e-12
        assert np.max(np.abs(g - r)) <= TC_GRAD_TOL * scale, (name, np.max(np.abs(g - r)) / scale)
        if size > 8:
            assert np.corrcoef(g, r)[0, 1] > TC_GRAD_CORR, name
        off += size


@pytest.mark.parametrize("seed,precision", [(5, 1), (6, 1), (5, 3), (6, 3), (5, 4), (6, 4)])
def test_bf16_tensor_core_inference_matches_fp32_forward(sph, gpu, seed, precision):
    """The inference kernels -- precision 1: the macro-step's default mma.sync kernels (BF16,
    FP32 accumulation); 3: the tcgen05 kernels (BF16 MMAs, FP32 accumulation in TMEM, f16 edge
    sums); 4: round 1 on tcgen05 with the features on the TMEM lanes, round 2 mma.sync --
    against the FP32 forward on the same frame: BF16 rounds weights and activations to 8
    mantissa bits, so the outputs agree to a few percent of their scale."""
    from oracle import mpnn_oracle as MO

    pos, vel, rho, nb, cnt, target, fc = random_frame(seed, n=200)
    n = len(pos)
    pos4 = np.zeros((n, 4), np.float32); pos4[:, :3] = pos
    vel4 = np.zeros((n, 4), np.float32); vel4[:, :3] = vel
    rhop = np.zeros((n, 2), np.float32); rhop[:, 0] = rho
    with sph.Net(256) as net:
        net.set_params(MO.init_params(seed))
        o32 = net.forward(pos4, vel4, rhop, nb, cnt, fc, precision=0)[:, :MO.FO]
        o16 = net.forward(pos4, vel4, rhop, nb, cnt, fc, precision=precision)[:, :MO.FO]
    scale = np.abs(o32).max()
    assert scale > 0
    err = np.abs(o16 - o32).max() / scale
    assert err < 0.05, err
    corr = np.corrcoef(o16.ravel(), o32.ravel())[0, 1]
    assert corr > 0.999, corr


# BF16 inference against the FP64 network on a frame recorded from the plain step: the
# outputs agree to INF_TOL of their scale element by element and to INF_RMS in RMS.
INF_TOL, INF_RMS, INF_CORR = 5e-2, 1.5e-2, 0.999
WEIGHTS = __import__("pathlib").Path(__file__).resolve().parents[1] / "npr-sph_gb300" / "weights" / "mpnn_w64.npy"


@pytest.mark.parametrize("steps,precision", [(8, 1), (60, 1), (8, 3), (60, 3), (8, 4), (60, 4)])
def test_tensor_core_inference_matches_fp64_oracle_on_dam_break(sph, gpu, steps, precision):
    """The BF16 inference kernels (precision 1: mma.sync, the macro-step's default; 3: tcgen05;
    4: tcgen05 round 1 with the features on the TMEM lanes, mma.sync round 2)
    with the committed trained weights, on the neighbour lists, densities and state of a
    16,384-particle dam break after `steps` plain steps, against oracle/mpnn_oracle.py in FP64
    on the same inputs."""
    from oracle import mpnn_oracle as MO

    if not WEIGHTS.exists():
        pytest.skip("no trained weights")
    w = np.load(WEIGHTS).astype(np.float32)
    sc = sph.dam_break(16, 32, 32, seed=41)
    p = sc.params
    with sph.Sim(p, n_max=len(sc.particles)) as sim:
        sim.upload(sc.particles)
        sim.step(steps)
        nb, cnt, rho = sim.neighbor_lists()
        rec = sim.download()
    n = len(rec)
    h = p.h
    c = float(np.sqrt(np.float32(p.gas_const)))
    rho_self = float(p.mass) * 315.0 / (64.0 * np.pi * h ** 3)
    fc = np.array([h, c, rho_self, p.resting_rho, np.log10(p.visc) / 4.0, c * p.dt / h], np.float32)
    pos4 = np.ascontiguousarray(rec["pos"], np.float32)
    vel4 = np.ascontiguousarray(rec["vel"], np.float32)
    rhop = np.zeros((n, 2), np.float32)
    rhop[:, 0] = rho
    assert cnt.max() > 16 and np.all(nb[np.arange(32)[None, :] >= cnt[:, None]] == -1)
    with sph.Net(n) as net:
        net.set_params(w)
        got = net.forward(pos4, vel4, rhop, nb, cnt, fc, precision=precision)[:, :MO.FO].astype(np.float64)
    f64 = lambda a: np.asarray(a, np.float32).astype(np.float64)
    e, mask, nf = MO.features(f64(pos4[:, :3]), f64(vel4[:, :3]), f64(rho), nb, cnt, *[float(x) for x in fc[:4]],
                              float(p.visc), float(fc[5]) * float(fc[0]) / float(fc[1]))
    ref, _ = MO.forward(w.astype(np.float64), e, mask, nf, nb)
    scale = np.abs(ref).max()
    assert np.abs(got - ref).max() <= INF_TOL * scale, np.abs(got - ref).max() / scale
    assert np.sqrt(np.mean((got - ref) ** 2)) <= INF_RMS * scale
    assert np.corrcoef(got.ravel(), ref.ravel())[0, 1] > INF_CORR


@pytest.fixture(scope="module")
def trained(sph, gpu):
    """A network trained briefly on frames of two small dam breaks (k and mu varied)."""
    from oracle import mpnn_oracle as MO

    net = sph.Net(20000)
    net.set_params(MO.init_params(0))
    for seed, k, mu in ((11, 2000.0, 3000.0), (12, 1200.0, 1.0)):
        sc = sph.dam_break(16, 32, 32, seed=seed, flags=sph.FLAG_KEEP_FORCE)
        p = sc.params.copy()
        p.gas_const, p.visc = k, mu
        with sph.Sim(p, n_max=len(sc.particles)) as sim:
            sim.upload(sc.particles)
            sim.step(8)
            net.record(sim, 6)
    losses = net.train(600, lr=2e-3, seed=1)
    yield net, losses
    net.close()


def test_training_reduces_the_loss(trained):
    _, losses = trained
    assert np.all(np.isfinite(losses))
    assert losses[-50:].mean() < 0.5 * losses[:20].mean()


def test_trained_network_beats_the_macro_step_without_it(sph, trained):
    from oracle import mpnn_oracle as MO

    net, _ = trained
    sc = sph.dam_break(16, 32, 32, seed=21)
    devs = {}
    with sph.Net(16) as zero:
        zero.set_params(np.zeros(MO.n_params(), np.float32))
        for name, nn in (("trained", net), ("zero", zero)):
            with sph.Sim(sc.params, n_max=len(sc.particles)) as sim:
                sim.upload(sc.particles)
                sim.step(8)
                rep = sim.learned_step(nn, 1, judge_every=1, density_tol=1.0, momentum_tol=1e9)
                assert rep.judged == 1 and rep.fallbacks == 0
                devs[name] = rep.last_density_dev
    assert devs["trained"] < devs["zero"], devs


def test_momentum_projection_conserves_momentum(sph, trained):
    """Away from the walls plain SPH changes the momentum only by gravity (pressure and
    viscosity are pairwise antisymmetric); the learned macro-step's projection makes the
    network's heads average G/A, so its momentum matches plain SPH to rounding."""
    net, _ = trained
    p = sph.workload_params(lower=(0.0, 0.0, 0.0), upper=(1.0, 1.0, 1.0))
    parts = sph.scene_ball(4000, (0.5, 0.5, 0.5), 0.5 * p.h, 0.01 * p.h, 31)
    with sph.Sim(p, n_max=len(parts)) as sim:
        sim.upload(parts)
        sim.step(8)
        rep = sim.learned_step(net, 1, judge_every=1, density_tol=1e30, momentum_tol=1e30)
    assert rep.judged == 1 and rep.learned_macro_steps == 1
    assert rep.last_momentum_dev < 2e-4, rep.last_momentum_dev


def test_judge_rolls_back_to_plain(sph, trained):
    """With zero tolerance every learned interval fails: it is rolled back to its checkpoint and
    run by plain SPH, and after the second failure in a row one more interval runs plain. The
    result is bit for bit the plain trajectory."""
    net, _ = trained
    sc = sph.dam_break(16, 32, 32, seed=22)
    with sph.Sim(sc.params, n_max=len(sc.particles)) as sim, \
            sph.Sim(sc.params, n_max=len(sc.particles)) as plain:
        for s in (sim, plain):
            s.upload(sc.particles)
            s.step(4)
        rep = sim.learned_step(net, 6, judge_every=2, density_tol=0.0, momentum_tol=0.0)
        assert (rep.judged, rep.fallbacks, rep.learned_macro_steps, rep.plain_macro_steps,
                rep.discarded_macro_steps) == (2, 2, 0, 6, 4)
        assert sim.steps == 4 + 6 * 4
        plain.step(24)
        a, b = sim.download(), plain.download()
        assert sim.reduce().nonfinite == 0
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])


def test_learned_run_stays_finite(sph, trained):
    net, _ = trained
    sc = sph.dam_break(16, 32, 32, seed=23)
    with sph.Sim(sc.params, n_max=len(sc.particles)) as sim:
        sim.upload(sc.particles)
        sim.step(4)
        rep = sim.learned_step(net, 16, judge_every=8, density_tol=0.05, momentum_tol=0.05)
        d = sim.reduce()
        out = sim.download()
    assert rep.judged == 2  # a first failure is retried at the next interval
    assert rep.learned_macro_steps + rep.plain_macro_steps == 16
    assert d.nonfinite == 0
    lo, hi = np.array(sc.params.lower[:3]), np.array(sc.params.upper[:3])
    assert np.all(out["pos"][:, :3] >= lo) and np.all(out["pos"][:, :3] <= hi)


def test_judge_metric_selects_the_density_deviation(sph, trained):
    """Both density deviations of a judged macro-step are reported and the selected one
    decides. The deviation of the mean density is far below the mean per-particle deviation,
    so a tolerance between the two keeps the learned interval under JUDGE_MEAN_DENSITY and
    rolls it back under JUDGE_PARTICLE_DENSITY, which a new context uses by default."""
    net, _ = trained
    sc = sph.dam_break(16, 32, 32, seed=24)
    out = {}
    with sph.Sim(sc.params, n_max=len(sc.particles)) as sim:
        sim.upload(sc.particles)
        sim.step(8)
        start = sim.download()
        probe = sim.learned_step(net, 1, 1, 1e30, 1e30)
        assert probe.judged == 1 and probe.learned_macro_steps == 1
        assert 0.0 <= probe.last_mean_rho_dev < 0.5 * probe.last_density_dev
        tol = 0.5 * (probe.last_mean_rho_dev + probe.last_density_dev)
        for metric in (sph.JUDGE_MEAN_DENSITY, sph.JUDGE_PARTICLE_DENSITY):
            sim.upload(start)
            sim.set_judge(metric)
            out[metric] = sim.learned_step(net, 1, 1, tol, 1e30)
        with pytest.raises(sph.SphError):
            sim.set_judge(7)
    with sph.Sim(sc.params, n_max=len(sc.particles)) as fresh:  # no set_judge: the default metric
        fresh.upload(start)
        default = fresh.learned_step(net, 1, 1, tol, 1e30)
    mean, part = out[sph.JUDGE_MEAN_DENSITY], out[sph.JUDGE_PARTICLE_DENSITY]
    assert (mean.learned_macro_steps, mean.fallbacks) == (1, 0)
    assert (part.learned_macro_steps, part.fallbacks) == (0, 1)
    assert (default.learned_macro_steps, default.fallbacks) == (0, 1)


def test_max_density_bound(sph, trained):
    """sph_learned_set_max_density_tol: the judge also fails an interval whose maximum density
    deviates from plain SPH's by more than the bound (unbounded by default)."""
    net, _ = trained
    sc = sph.dam_break(16, 32, 32, seed=25)
    with sph.Sim(sc.params, n_max=len(sc.particles)) as sim:
        sim.upload(sc.particles)
        sim.step(8)
        start = sim.download()
        probe = sim.learned_step(net, 1, 1, 1e30, 1e30)
        assert probe.learned_macro_steps == 1 and probe.last_max_rho_dev > 0.0
        out = {}
        for name, tol in (("tight", 0.5 * probe.last_max_rho_dev), ("loose", 2.0 * probe.last_max_rho_dev + 1e-6)):
            sim.upload(start)
            sim.set_max_density_tol(tol)
            out[name] = sim.learned_step(net, 1, 1, 1e30, 1e30)
        with pytest.raises(sph.SphError):
            sim.set_max_density_tol(-1.0)
    assert (out["tight"].learned_macro_steps, out["tight"].fallbacks) == (0, 1)
    assert (out["loose"].learned_macro_steps, out["loose"].fallbacks) == (1, 0)


def test_rollout_rounds_record_states_the_network_reached(sph, trained):
    """train_mpnn's rollout round on two small runs: frames recorded after unjudged learned
    macro-steps of the current network (plain steps first), then Adam over plain and rollout
    frames from the current weights: the frame count, a finite loss and changed weights."""
    import train_mpnn as TM

    net, _ = trained
    before = net.get_params()
    plist, counts, parts = TM.training_scenes(2, 4096, seed=7)
    net.clear_frames()
    with sph.Sim(plist, counts=counts) as sim:
        sim.upload(parts)
        n_plain = net.record(sim, 2)
    assert n_plain == 4
    total = TM.rollout_frames(net, plist, counts, parts, per_run=3, macro=4, seed=1)
    assert total == n_plain + 2 * 3
    losses = TM.train_steps(net, 200, 3e-4, seed=2)
    assert losses.shape == (200,) and np.all(np.isfinite(losses))
    assert not np.array_equal(net.get_params(), before)
    net.set_params(before)
