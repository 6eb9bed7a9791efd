"""Neighbour sets of the GPU grid are bit-exact against brute force (the reference's
all-pairs j-loop, rho_pres_comp.glsl:46-50) on the same FP32 positions: counts and
order-independent digests sum_j mix64(j) agree exactly."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def queries(n, k, seed):
    return np.sort(np.random.default_rng(seed).choice(n, size=min(k, n), replace=False)).astype(np.uint32)


def test_dam_break_1m_subsample_vs_gpu_brute_and_oracle(sph, orc, gpu):
    """1,048,576-particle dam break: 65,536 seeded query particles against all N, at the start
    and after 40 steps (the block has begun to spread)."""
    sc = sph.dam_break()
    q = queries(len(sc.particles), 65536, 1)
    with sph.Sim(sc.params, n_max=len(sc.particles)) as sim:
        sim.upload(sc.particles)
        for steps in (0, 40):
            sim.step(steps)
            cg, dg = sim.neighbor_digest(q, brute_force=False)
            cb, db = sim.neighbor_digest(q, brute_force=True)
            np.testing.assert_array_equal(cg, cb)
            np.testing.assert_array_equal(dg, db)
            state = sim.download()
            co, do = orc.neighbors(sc.params, state, q, backend="grid")
            np.testing.assert_array_equal(cg, co)
            np.testing.assert_array_equal(dg, do)
            assert cg.min() >= 1 and cg.mean() > 5


def test_subscene_65536_against_cpu_brute_force(sph, orc, gpu):
    """A 65,536-particle dam break, every particle checked against the oracle's brute force."""
    sc = sph.dam_break(16, 64, 64, seed=12)
    n = len(sc.particles)
    q = np.arange(n, dtype=np.uint32)
    with sph.Sim(sc.params, n_max=n) as sim:
        sim.upload(sc.particles)
        sim.step(25)
        cg, dg = sim.neighbor_digest(q)
        state = sim.download()
    co, do = orc.neighbors(sc.params, state, q, backend="brute")
    np.testing.assert_array_equal(cg, co)
    np.testing.assert_array_equal(dg, do)


@pytest.mark.parametrize("stencil", [1, 2])
def test_edge_cases(sph, orc, gpu, stencil):
    """Walls, positions beyond the walls (before the first clamp), coincident particles and
    pairs at exactly r = h, for both cell sizes."""
    p = sph.default_params()
    h = np.float32(p.h)
    lo, hi = np.array(p.lower[:3], np.float32), np.array(p.upper[:3], np.float32)
    rng = np.random.default_rng(5)
    pos = rng.uniform(lo, hi, (6000, 3)).astype(np.float32)
    pos[:500, 0] = lo[0]
    pos[500:1000, 2] = hi[2]
    pos[1000:1200] = pos[1200:1400]
    pos[1400:1500, 1] = hi[1] + rng.uniform(0, 4 * h, 100)
    g = (np.stack(np.meshgrid(*[np.arange(10)] * 3, indexing="ij"), -1).reshape(-1, 3) * h + lo + 0.05)
    pos[2000:3000] = g.astype(np.float32)
    a = sph.empty_particles(len(pos))
    a["pos"][:, :3] = pos
    a["pos"][:, 3] = 1
    q = np.arange(len(a), dtype=np.uint32)
    with sph.Sim(p, n_max=len(a)) as sim:
        sim.set_launch(256, stencil)
        sim.upload(a)
        cg, dg = sim.neighbor_digest(q)
        cb, db = sim.neighbor_digest(q, brute_force=True)
    co, do = orc.neighbors(p, a, q, backend="brute")
    np.testing.assert_array_equal(cg, co)
    np.testing.assert_array_equal(dg, do)
    np.testing.assert_array_equal(cb, co)
    np.testing.assert_array_equal(db, do)


def _rod(sph):
    """Particles ~31 per cell in one cell row: row segments longer than one pair mask."""
    p = sph.workload_params(lower=(0.0, 0.0, 0.0), upper=(3.6, 0.3, 0.3))
    s = p.h / 3.5
    lo = (0.01, 0.1015, 0.1015)
    return p, sph.scene_fill(600 * 9, lo, (lo[0] + 600.5 * s, lo[1] + 3.2 * s, lo[2] + 3.2 * s), s, 0.01 * p.h, 12)


def _pile_up(sph):
    """A clump denser than a shared-memory tile holds next to a lattice: the global-memory path."""
    p = sph.default_params()
    rng = np.random.default_rng(3)
    pos = np.concatenate([0.2 + rng.uniform(-p.h, p.h, (4000, 3)),
                          sph.reference_scene_10k(seed=5).particles["pos"][:6000, :3]])
    a = sph.empty_particles(len(pos))
    a["pos"][:, :3] = pos
    a["pos"][:, 3] = 1
    return p, a


@pytest.mark.parametrize("scene", ["dam_break", "long_segments", "pile_up"])
@pytest.mark.parametrize("block", [256, 128])
def test_force_pass_neighbour_sets(sph, gpu, scene, block):
    """The neighbour sets the force pass interacts with -- decoded from the density pass's pair
    masks, tested by the force pass itself in over-long segments, or on the global-memory path
    -- equal brute force on the positions before the step, bit for bit (counts and digests)."""
    if scene == "dam_break":
        sc = sph.dam_break(32, 64, 64, seed=8)
        p, parts, warm = sc.params, sc.particles, 20
    elif scene == "long_segments":
        (p, parts), warm = _rod(sph), 0
    else:
        (p, parts), warm = _pile_up(sph), 0
    q = queries(len(parts), 16384, 2)
    with sph.Sim(p, n_max=len(parts)) as sim:
        sim.set_launch(block, 1)
        sim.upload(parts)
        sim.step(warm)
        for _ in range(2):
            cb, db = sim.neighbor_digest(q, brute_force=True)
            cf, df = sim.step_neighbor_digest(q)
            np.testing.assert_array_equal(cf, cb)
            np.testing.assert_array_equal(df, db)
        fb = sim.tile_stats()
    assert cb.min() >= 1
    if scene == "pile_up":
        assert fb[1] > 0  # chunks on the global-memory path took part
    with sph.Sim(p, n_max=len(parts)) as sim:
        sim.set_launch(block, 2)
        sim.upload(parts)
        with pytest.raises(sph.SphError):
            sim.step_neighbor_digest(q)


def test_batched_neighbours(sph, orc, gpu):
    plist, counts, parts = sph.batched_scenes(8, seed=31, n_lo=2000, n_hi=8000)
    offs = np.concatenate([[0], np.cumsum(counts, dtype=np.int64)])
    q = np.arange(len(parts), dtype=np.uint32)
    with sph.Sim(plist, counts=counts) as sim:
        sim.upload(parts)
        sim.step(10)
        cg, dg = sim.neighbor_digest(q)
        cb, db = sim.neighbor_digest(q, brute_force=True)
        state = sim.download()
    np.testing.assert_array_equal(cg, cb)
    np.testing.assert_array_equal(dg, db)
    for i, p in enumerate(plist):
        seg = state[offs[i]:offs[i + 1]]
        co, _ = orc.neighbors(p, seg, np.arange(len(seg)), backend="grid")
        np.testing.assert_array_equal(cg[offs[i]:offs[i + 1]], co)


@pytest.mark.gpu
@pytest.mark.parametrize("scene,steps", [("reference_grid", 0), ("dam_break", 150)])
def test_nearest_32_lists_against_brute_force(sph, orc, gpu, scene, steps):
    """The learned macro-step's input (sph_neighbor_lists): per particle the <= 32 nearest
    neighbours j != i with r < h. Against the brute-force oracle lists, compared as multisets
    of FP32 canonical distances (ties may pick either particle); the density equals the plain
    density pass bit for bit. The reference's own start (make_grid: 0.25h lattice, ~180
    neighbours, chunks too dense for a shared-memory tile) exercises the nearest-32 selection
    on both paths; a 0.5h lattice holds at most 32 neighbours, so the dam break after 150
    steps covers the ordinary case."""
    if scene == "reference_grid":
        params, parts = sph.default_params(), sph.scene_reference_grid()
    else:
        sc = sph.dam_break(16, 32, 32, seed=41)
        params, parts = sc.params, sc.particles
    with sph.Sim(params, n_max=len(parts)) as sim:
        sim.upload(parts)
        sim.step(steps)
        state = sim.download()
        nb, cnt, rho = sim.neighbor_lists()
        sim.refresh_density()
        rho_plain = sim.download()["extras"][:, 0]
    assert np.array_equal(rho, rho_plain)
    pos = np.ascontiguousarray(state["pos"][:, :3], dtype=np.float32)
    off, items = orc.neighbor_lists(params, state, backend="brute")

    def d2(i, js):
        d = pos[js] - pos[i]
        return (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]

    n = len(pos)
    over = 0
    for i in range(n):
        ref = items[off[i]:off[i + 1]]
        ref = ref[ref != i]
        k = min(len(ref), 32)
        over += len(ref) > 32
        assert cnt[i] == k, (i, cnt[i], len(ref))
        got = nb[i, :k]
        assert np.all(nb[i, k:] == -1)
        assert np.all(np.isin(got, ref)) and len(np.unique(got)) == k
        assert np.array_equal(np.sort(d2(i, got)), np.sort(d2(i, ref))[:k])
    if scene == "reference_grid":
        assert over > n // 2  # the dense lattice exercises the nearest-32 selection
