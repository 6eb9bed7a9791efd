"""GPU step vs the FP64 oracle, one step at a time from the GPU's own state (the step is
chaotic, so trajectories are not compared; every step is). All calls go through the C ABI."""
from __future__ import annotations

import numpy as np
import pytest

from gpu_helpers import check_step

pytestmark = pytest.mark.gpu


def run_parity(sph, orc, params, parts, steps, launch=None, stride=1):
    params = params.copy()
    params.flags |= sph.FLAG_KEEP_FORCE
    with sph.Sim(params, n_max=len(parts)) as sim:
        if launch:
            sim.set_launch(*launch)
        sim.upload(parts)
        state = sim.download()
        errs = []
        for s in range(steps):
            sim.step(1)
            after = sim.download()
            if s % stride == 0:
                errs.append(check_step(orc, params, state, after))
            state = after
        sim.synchronize()
    return errs


def tiny(sph, pos, vel=None):
    a = sph.empty_particles(len(pos))
    a["pos"][:, :3] = np.asarray(pos, np.float32)
    a["pos"][:, 3] = 1.0
    if vel is not None:
        a["vel"][:, :3] = np.asarray(vel, np.float32)
    return a


def test_isolated_and_small_clusters(sph, orc, gpu):
    p = sph.default_params()
    h = p.h
    run_parity(sph, orc, p, tiny(sph, [[0.2, 0.3, 0.2]]), 3)
    run_parity(sph, orc, p, tiny(sph, [[0.2, 0.3, 0.2], [0.2 + 0.5 * h, 0.3, 0.2]]), 3)
    rng = np.random.default_rng(0)
    pos = 0.2 + rng.uniform(-1.5 * h, 1.5 * h, (27, 3))
    run_parity(sph, orc, p, tiny(sph, pos, rng.normal(0, 0.1, (27, 3))), 5)


def test_coincident_pair_is_finite(sph, orc, gpu):
    p = sph.default_params()
    a = tiny(sph, [[0.2, 0.3, 0.2], [0.2, 0.3, 0.2], [0.2 + 0.3 * p.h, 0.3, 0.2]])
    errs = run_parity(sph, orc, p, a, 2)
    assert errs


def test_reference_literal_scene(sph, orc, gpu):
    """make_grid() start (0.25h lattice, ~180 neighbours) with the shaders' own constants."""
    run_parity(sph, orc, sph.default_params(), sph.scene_reference_grid(), 5)


def test_reference_scene_10k_200_steps(sph, orc, gpu):
    """10,000 particles, 0.5h jittered lattice, g = -9.81, 200 steps, every step checked."""
    sc = sph.reference_scene_10k(seed=1)
    errs = run_parity(sph, orc, sc.params, sc.particles, sc.steps)
    assert len(errs) == 200


@pytest.mark.parametrize("launch", [(256, 1), (128, 1), (256, 2), (128, 2)])
def test_dam_break_crop(sph, orc, gpu, launch):
    sc = sph.dam_break(32, 64, 64, seed=4)
    run_parity(sph, orc, sc.params, sc.particles, 6, launch=launch)


@pytest.mark.parametrize("stencil", [1, 2])
def test_pile_up_takes_the_global_path(sph, orc, gpu, stencil):
    """A clump far denser than a shared-memory tile holds (4,000 particles in a 2h cube)
    next to an ordinary lattice: its chunks read neighbours from global memory, with the
    same results."""
    p = sph.default_params()
    h = p.h
    rng = np.random.default_rng(3)
    clump = 0.2 + rng.uniform(-h, h, (4000, 3))
    lattice = sph.reference_scene_10k(seed=5).particles["pos"][:6000, :3]
    a = tiny(sph, np.concatenate([clump, lattice]))
    pp = p.copy()
    pp.flags |= sph.FLAG_KEEP_FORCE
    with sph.Sim(pp, n_max=len(a)) as sim:
        sim.set_launch(256, stencil)
        sim.upload(a)
        sim.step(1)
        after = sim.download()
        fb = sim.tile_stats()
    check_step(orc, pp, a, after)
    assert fb[0] > 0 and fb[1] > 0


@pytest.mark.parametrize("block", [256, 128])
def test_long_segments_in_a_tile(sph, orc, gpu, block):
    """A rod of particles one cell thick in y and z, at spacing h/3.5 (~31 per cell): each
    particle's own 3-cell row segment holds ~90 candidates, more than the 32 candidate pairs of
    one pair mask, while every chunk fits the shared-memory tile (the neighbour rows are
    empty). The force pass then tests that segment itself instead of reading the density
    pass's masks; results as elsewhere."""
    p = sph.workload_params(lower=(0.0, 0.0, 0.0), upper=(3.6, 0.3, 0.3))
    s = p.h / 3.5
    lo = (0.01, 0.1015, 0.1015)  # y and z inside cell 5 (cell edge h (1 + 2^-10))
    parts = sph.scene_fill(600 * 3 * 3, lo, (lo[0] + 600.5 * s, lo[1] + 3.2 * s, lo[2] + 3.2 * s), s,
                           0.01 * p.h, 12)
    edge = p.h * (1.0 + 2.0 ** -10)
    c = np.floor(parts["pos"][:, :3].astype(np.float64) / edge).astype(np.int64)
    assert np.all(c[:, 1] == 5) and np.all(c[:, 2] == 5)
    occ = np.bincount(c[:, 0])
    seg = occ[c[:, 0]] + occ[np.maximum(c[:, 0] - 1, 0)] * (c[:, 0] > 0) + \
        np.append(occ, 0)[c[:, 0] + 1]
    assert (seg > 64).mean() > 0.9  # candidates of the particle's own row segment
    pp = p.copy()
    pp.flags |= sph.FLAG_KEEP_FORCE
    with sph.Sim(pp, n_max=len(parts)) as sim:
        sim.set_launch(block, 1)
        sim.upload(parts)
        sim.step(1)
        after = sim.download()
        fb = sim.tile_stats()
    check_step(orc, pp, parts, after)
    assert fb == (0, 0), fb  # every chunk took the tile (and the masks)


def test_upload_download_roundtrip(sph, gpu):
    sc = sph.reference_scene_10k(seed=2)
    a = sc.particles.copy()
    rng = np.random.default_rng(1)
    a["vel"] = rng.normal(size=(len(a), 4)).astype(np.float32)
    a["force"] = rng.normal(size=(len(a), 4)).astype(np.float32)
    a["extras"] = rng.normal(size=(len(a), 4)).astype(np.float32)
    with sph.Sim(sc.params, n_max=len(a) + 5) as sim:
        sim.upload(a)
        b = sim.download()
        np.testing.assert_array_equal(a.view(np.uint8), b.view(np.uint8))
        sim.step(3)
        c = sim.download()
        # untouched fields come back as uploaded
        np.testing.assert_array_equal(c["pos"][:, 3], a["pos"][:, 3])
        np.testing.assert_array_equal(c["vel"][:, 3], a["vel"][:, 3])
        np.testing.assert_array_equal(c["extras"][:, 2:], a["extras"][:, 2:])
        np.testing.assert_array_equal(c["force"], a["force"])  # KEEP_FORCE off


def test_chunked_host_transfers(sph, gpu):
    """Host uploads and downloads of more than 4 x 65,536 records move in four uneven chunks on a
    transfer stream (records assembled by particle id); device-buffer transfers take one pass by
    slot. Both give the same bytes, before and after steps, with and without kept forces."""
    import torch

    p = sph.workload_params(lower=(0.0, 0.0, 0.0), upper=(1.6, 1.6, 1.6))
    n = 4 * 65536 + 3
    parts = sph.scene_fill(n, (0.02, 0.02, 0.02), (1.58, 1.0, 1.58), 0.5 * p.h, 0.01 * p.h, 21)
    rng = np.random.default_rng(4)
    parts["vel"][:, :3] = rng.normal(0.0, 0.2, (n, 3)).astype(np.float32)
    parts["vel"][:, 3] = rng.normal(size=n).astype(np.float32)
    parts["force"] = rng.normal(size=(n, 4)).astype(np.float32)
    parts["extras"][:, 2:] = rng.normal(size=(n, 2)).astype(np.float32)
    for flags in (0, sph.FLAG_KEEP_FORCE):
        pp = p.copy()
        pp.flags |= flags
        with sph.Sim(pp, n_max=n) as sim:
            sim.upload(parts)
            np.testing.assert_array_equal(sim.download().view(np.uint8), parts.view(np.uint8))
            dev = torch.empty(n * 64, dtype=torch.uint8, device=gpu)
            for steps in (1, 3):
                sim.step(steps)
                host = sim.download()
                sim.download_device(dev.data_ptr(), n)
                sim.synchronize()
                np.testing.assert_array_equal(host.view(np.uint8), dev.cpu().numpy())
            sim.upload(host)  # a chunked upload of the stepped records, then one more step
            sim.step(1)
            again = sim.download()
            assert np.isfinite(again["pos"][:, :3]).all()


def test_device_aos_buffers(sph, gpu):
    import torch

    sc = sph.reference_scene_10k(seed=3)
    n = len(sc.particles)
    dev = torch.from_numpy(sc.particles.view(np.uint8).copy()).to(gpu)
    with sph.Sim(sc.params, n_max=n) as a, sph.Sim(sc.params, n_max=n) as b:
        a.upload(sc.particles)
        torch.cuda.synchronize()
        b.upload_device(dev.data_ptr(), n)
        a.step(4)
        b.step(4)
        b.download_device(dev.data_ptr(), n)
        b.synchronize()
        got = dev.cpu().numpy().view(sph.PARTICLE_DTYPE)
        np.testing.assert_array_equal(got.view(np.uint8), a.download().view(np.uint8))


def test_deterministic(sph, gpu):
    sc = sph.dam_break(32, 64, 64, seed=6)
    outs = []
    for _ in range(2):
        with sph.Sim(sc.params, n_max=len(sc.particles)) as sim:
            sim.upload(sc.particles)
            sim.step(20)
            outs.append(sim.download())
    np.testing.assert_array_equal(outs[0].view(np.uint8), outs[1].view(np.uint8))


def test_neighbour_record_forms_are_bit_identical(sph, gpu):
    """The force pass reads each neighbour either as the density pass's 32-byte record or from
    the state arrays; both compute the same interactions from the same values, so the
    trajectories agree bit for bit over the dense start and the expansion of a dam break, and
    the per-step choice (auto) agrees with both."""
    sc = sph.dam_break(32, 64, 64, seed=6)
    outs, stats = [], []
    for mode in (sph.RECORDS_ALWAYS, sph.RECORDS_NEVER, sph.RECORDS_AUTO):
        with sph.Sim(sc.params, n_max=len(sc.particles)) as sim:
            sim.set_record_mode(mode)
            sim.upload(sc.particles)
            for _ in range(10):
                sim.step(50)
                sim.synchronize()
            outs.append(sim.download())
            stats.append(sim.record_stats())
    assert stats[0][:2] == (500, 0) and stats[1][:2] == (0, 500)
    assert stats[2][0] > 0 and stats[2][1] > 0, stats[2]  # dense start with, expansion without
    np.testing.assert_array_equal(outs[0].view(np.uint8), outs[1].view(np.uint8))
    np.testing.assert_array_equal(outs[2].view(np.uint8), outs[1].view(np.uint8))
    with sph.Sim(sc.params, n_max=len(sc.particles)) as sim:
        with pytest.raises(sph.SphError):
            sim.set_record_mode(3)


def test_batched_matches_single_scenes(sph, orc, gpu):
    """A scene stepped inside a batch equals the same scene stepped alone up to FP32 rounding
    (not bit for bit: the packed pair lanes of the density sum follow where a row segment lands
    in shared memory, which depends on the neighbouring scenes)."""
    plist, counts, parts = sph.batched_scenes(12, seed=9, n_lo=500, n_hi=6000)
    offs = np.concatenate([[0], np.cumsum(counts, dtype=np.int64)])
    with sph.Sim(plist, counts=counts) as bat:
        bat.upload(parts)
        bat.step(1)
        got = bat.download()
        diags = bat.reduce_scenes()
    for i, p in enumerate(plist):
        seg = parts[offs[i]:offs[i + 1]]
        with sph.Sim(p, n_max=len(seg)) as one:
            one.upload(seg)
            one.step(1)
            ref = one.download()
            d1 = one.reduce()
        g = got[offs[i]:offs[i + 1]]
        np.testing.assert_allclose(g["extras"][:, 0], ref["extras"][:, 0], rtol=1e-6)
        np.testing.assert_allclose(g["pos"][:, :3], ref["pos"][:, :3], rtol=0, atol=1e-6)
        assert diags[i].n == len(seg)
        assert diags[i].mean_rho == pytest.approx(d1.mean_rho, rel=1e-6)


def test_batched_parity_per_scene(sph, orc, gpu):
    plist, counts, parts = sph.batched_scenes(6, seed=21, n_lo=1000, n_hi=4000)
    plist = [p.copy() for p in plist]
    for p in plist:
        p.flags |= sph.FLAG_KEEP_FORCE
    offs = np.concatenate([[0], np.cumsum(counts, dtype=np.int64)])
    with sph.Sim(plist, counts=counts) as bat:
        bat.upload(parts)
        state = bat.download()
        for _ in range(3):
            bat.step(1)
            after = bat.download()
            for i, p in enumerate(plist):
                check_step(orc, p, state[offs[i]:offs[i + 1]], after[offs[i]:offs[i + 1]])
            state = after


def test_set_params_between_steps(sph, orc, gpu):
    sc = sph.reference_scene_10k(seed=4)
    p = sc.params.copy()
    p.flags |= sph.FLAG_KEEP_FORCE
    with sph.Sim(p, n_max=len(sc.particles)) as sim:
        sim.upload(sc.particles)
        sim.step(2)
        p2 = p.copy()
        p2.gas_const, p2.visc, p2.smoothing_coeff = 900.0, 1.5, 4.5
        sim.set_params(p2)
        before = sim.download()
        sim.step(1)
        check_step(orc, p2, before, sim.download())


def test_reduce_matches_host_fp64(sph, gpu):
    sc = sph.dam_break(32, 64, 64, seed=8)
    with sph.Sim(sc.params, n_max=len(sc.particles)) as sim:
        sim.upload(sc.particles)
        sim.step(5)
        d = sim.reduce()
        a = sim.download()
    m = float(np.float32(sc.params.mass))
    v = a["vel"][:, :3].astype(np.float64)
    rho = a["extras"][:, 0].astype(np.float64)
    np.testing.assert_allclose(d.momentum, m * v.sum(0), rtol=1e-9, atol=1e-12)
    assert d.kinetic_energy == pytest.approx(0.5 * m * (v * v).sum(), rel=1e-9)
    assert d.mean_rho == pytest.approx(rho.mean(), rel=1e-12)
    assert d.min_rho == rho.min() and d.max_rho == rho.max()
    assert d.nonfinite == 0 and d.n == len(a) and d.step == 5


def test_errors(sph, gpu):
    p = sph.default_params()
    with sph.Sim(p, n_max=100) as sim:
        with pytest.raises(sph.SphError) as e:
            sim.step(1)
        assert e.value.code == sph.ERR_NOT_READY
        with pytest.raises(sph.SphError) as e:
            sim.upload(sph.empty_particles(101))
        assert e.value.code == sph.ERR_CAPACITY
        sim.upload(sph.empty_particles(10))
        with pytest.raises(sph.SphError):
            sim.download(sph.empty_particles(11))
        with pytest.raises(sph.SphError):
            sim.set_launch(100, 1)


def test_timing_and_autotune(sph, orc, gpu):
    sc = sph.dam_break(32, 64, 64, seed=10)
    p = sc.params.copy()
    p.flags |= sph.FLAG_KEEP_FORCE
    with sph.Sim(p, n_max=len(sc.particles)) as sim:
        sim.upload(sc.particles)
        sim.enable_timing(True)
        sim.step(2)
        t = sim.pass_times()
        assert all(x > 0 for x in t)
        sim.enable_timing(False)
        start = sim.download()
        ms = sim.autotune(3)
        assert ms > 0
        blk, sten = sim.get_launch()
        assert blk in (128, 256) and sten in (1, 2)
        assert sim.steps == 2  # the state the autotuner started from is restored
        before = sim.download()
        np.testing.assert_array_equal(before["pos"], start["pos"])
        np.testing.assert_array_equal(before["vel"], start["vel"])
        sim.step(1)
        check_step(orc, p, before, sim.download())
