"""Static obstacles on the GPU: the mesh signed distance field (sph_sdf_from_mesh) against its
FP64 restatement, one step with an obstacle against the FP64 oracle step followed by the
oracle's obstacle rule, particles kept out of a sphere over a run (plain and learned), and the
argument checks and removal of sph_set_obstacle."""
from __future__ import annotations

import numpy as np
import pytest

from gpu_helpers import TOL, force_bound

pytestmark = pytest.mark.gpu


def sphere_sdf(n: int, spacing: float, center, radius: float) -> np.ndarray:
    g = np.arange(n) * spacing
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    return (np.sqrt((x - center[0]) ** 2 + (y - center[1]) ** 2 + (z - center[2]) ** 2) - radius).astype(np.float32)


def test_sdf_from_mesh_matches_restatement(sph, orc, gpu):
    v, t = sph.icosphere(0.1, (0.25, 0.22, 0.27), 2)
    dims, origin, spacing = (21, 18, 16), (0.05, 0.04, 0.08), 0.0213
    sdf = sph.sdf_from_mesh(v, t, dims, origin, spacing)
    assert sdf.shape == (16, 18, 21)
    z, y, x = np.meshgrid(*(origin[a] + spacing * np.arange(dims[a], dtype=np.float32) for a in (2, 1, 0)),
                          indexing="ij")
    pts = np.stack([x, y, z], -1).reshape(-1, 3).astype(np.float64)
    ref = orc.mesh_sdf(v, t, pts).reshape(sdf.shape)
    assert np.max(np.abs(np.abs(sdf) - np.abs(ref))) < 2e-6  # FP32 distances to FP64 ones
    sure = np.abs(ref) > 1e-4  # the winding number's 1/2 threshold is exact away from the surface
    assert np.array_equal(np.sign(sdf[sure]), np.sign(ref[sure]))
    assert (sdf < 0).sum() > 100 and (sdf > 0).sum() > 100


def inclined_floor(params, n_s: int = 17, spacing: float = 0.02):
    """Samples of the plane phi(x) = (x - x0) . nhat through the box: the trilinear interpolant of
    a linear field is exact and its sampled gradient is constant, so the rule's normal does not
    depend on which sample cell an FP32 or FP64 position falls into."""
    nhat = np.array([-0.3, 1.0, 0.2])
    nhat /= np.linalg.norm(nhat)
    x0 = np.array([0.15, 0.08, 0.15])
    g = np.arange(n_s) * spacing
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    sdf = ((x - x0[0]) * nhat[0] + (y - x0[1]) * nhat[1] + (z - x0[2]) * nhat[2]).astype(np.float32)
    return sdf, (0.0, 0.0, 0.0), spacing, nhat


def check_obstacle_step(orc, params, sdf, origin, spacing, before, after) -> int:
    """One GPU step with the obstacle against the oracle's force/integrate (from the GPU's own
    densities, as gpu_helpers.check_step does) followed by the oracle's obstacle rule. Where the
    oracle's phi at the integrated position is within 1e-5 of zero, FP32 and FP64 may disagree on
    whether the rule fires: such particles match either outcome. Returns how many particles the
    rule moved."""
    g_rho = after["extras"][:, 0].astype(np.float64)
    g_pres = after["extras"][:, 1].astype(np.float64)
    o = orc.force_f64(params, before, g_rho, g_pres)
    fb = force_bound(o, TOL)
    v_in = before["vel"][:, :3].astype(np.float64)
    vb = TOL * np.abs(v_in).max(axis=1) + params.dt * fb / g_rho
    xb = 2e-6 * (1.0 + np.abs(o["pos"]).max(axis=1)) + params.dt * vb
    xo, vo, phi = orc.obstacle_f64(params, sdf, origin, spacing, o["pos"], o["vel"])
    gx = after["pos"][:, :3].astype(np.float64)
    gv = after["vel"][:, :3].astype(np.float64)
    walls = o["margin"] <= 2e-6 * (1.0 + np.abs(o["pos"]).max(axis=1))  # covered by check_step
    amb = (np.abs(phi) <= 1e-5) & ~walls
    ok = ~amb & ~walls
    # the rule moves x by -phi n: position errors pass through, velocity errors too (n is exact)
    ex = np.abs(gx - xo).max(axis=1) / (2.0 * xb + 1e-7)
    ev = np.abs(gv - vo).max(axis=1) / (2.0 * vb + 1e-6)
    assert ex[ok].max() <= 1.0, ("pos", ex[ok].max())
    assert ev[ok].max() <= 1.0, ("vel", ev[ok].max())
    if amb.any():
        fired = (np.abs(gx - xo).max(axis=1) <= 2.0 * xb + 1e-7) & (np.abs(gv - vo).max(axis=1) <= 2.0 * vb + 1e-6)
        plain = (np.abs(gx - o["pos"]).max(axis=1) <= 2.0 * xb + 1e-7) & \
            (np.abs(gv - o["vel"]).max(axis=1) <= 2.0 * vb + 1e-6)
        assert np.all((fired | plain)[amb])
    return int(((phi < -1e-5) & ok).sum())


def test_obstacle_step_parity_with_oracle(sph, orc, gpu):
    p = sph.workload_params(lower=(0.0, 0.0, 0.0), upper=(0.32, 0.32, 0.32))
    p.flags |= sph.FLAG_KEEP_FORCE
    parts = sph.scene_fill(7000, (0.06, 0.02, 0.06), (0.26, 0.2, 0.26), 0.5 * p.h, 0.01 * p.h, 17)
    parts["vel"][:, 1] = -1.5
    parts["vel"][:, 0] = 0.4
    sdf, origin, spacing, _ = inclined_floor(p)
    moved = []
    with sph.Sim(p, n_max=len(parts)) as sim:
        sim.upload(parts)
        sim.set_obstacle(sdf, origin, spacing)
        done = 0
        for target in (0, 3, 20):
            sim.step(target - done)
            done = target
            before = sim.download()
            sim.step(1)
            done += 1
            after = sim.download()
            moved.append(check_obstacle_step(orc, p, sdf, origin, spacing, before, after))
    assert moved[0] > 100, moved  # the lattice starts partly below the floor: the rule fires


def test_particles_stay_out_of_a_sphere(sph, gpu):
    """A block of fluid falls onto a sampled sphere: after 300 steps no particle is inside it
    by more than the distance one step can carry it (the rule runs once per step), plain and
    with the learned macro-step (zero network: the rule runs after its update too)."""
    from oracle import mpnn_oracle as MO

    p = sph.workload_params(lower=(0.0, 0.0, 0.0), upper=(0.4, 0.4, 0.4))
    n_s, spacing = 41, 0.01
    center, radius = (0.2, 0.12, 0.2), 0.07
    sdf = sphere_sdf(n_s, spacing, center, radius)
    parts = sph.scene_fill(4000, (0.1, 0.22, 0.1), (0.3, 0.34, 0.3), 0.5 * p.h, 0.01 * p.h, 5)
    parts["vel"][:, 1] = -2.0

    def depth(out):
        return radius - np.linalg.norm(out["pos"][:, :3].astype(np.float64) - center, axis=1)

    with sph.Sim(p, n_max=len(parts)) as sim:
        sim.upload(parts)
        sim.set_obstacle(sdf, (0.0, 0.0, 0.0), spacing)
        hit = 0
        for _ in range(30):
            sim.step(10)
            out = sim.download()
            vmax = np.abs(out["vel"][:, :3]).max()
            d = depth(out)
            assert d.max() <= vmax * p.dt + 2e-3, (d.max(), vmax)  # inside by at most one step + sampling
            hit += int((d > -0.5 * p.h).sum())
        assert hit > 0  # the fluid reached the sphere
        assert sim.reduce().nonfinite == 0
        with sph.Net(16) as zero:
            zero.set_params(np.zeros(MO.n_params(), np.float32))
            sim.learned_step(zero, 8, 0)
        out = sim.download()
        vmax = np.abs(out["vel"][:, :3]).max()
        assert depth(out).max() <= 4 * vmax * p.dt + 2e-3


def test_set_obstacle_arguments_and_removal(sph, gpu):
    p = sph.workload_params(lower=(0.0, 0.0, 0.0), upper=(0.3, 0.3, 0.3))
    parts = sph.scene_fill(3000, (0.05, 0.05, 0.05), (0.25, 0.2, 0.25), 0.5 * p.h, 0.01 * p.h, 9)
    sdf = sphere_sdf(16, 0.02, (0.15, 0.1, 0.15), 0.05)
    with sph.Sim(p, n_max=len(parts)) as a, sph.Sim(p, n_max=len(parts)) as b:
        for bad in (dict(sdf=np.zeros((1, 4, 4), np.float32)), dict(sdf=sdf, spacing=0.0),
                    dict(sdf=sdf, origin=(np.nan, 0.0, 0.0))):
            kw = dict(origin=(0.0, 0.0, 0.0), spacing=0.02)
            kw.update(bad)
            with pytest.raises(sph.SphError):
                a.set_obstacle(kw.pop("sdf"), **kw)
        a.upload(parts)
        b.upload(parts)
        a.set_obstacle(sdf, (0.0, 0.0, 0.0), 0.02)
        a.step(5)
        a.set_obstacle(None)  # removed: the same plain step as a context that never had one
        b.step(5)
        sa, sb = a.download(), b.download()
        a.upload(sb)
        b.upload(sb)
        a.step(7)
        b.step(7)
        assert np.array_equal(a.download()["pos"], b.download()["pos"])
    assert not np.array_equal(sa["pos"], sb["pos"])  # the obstacle did act


def test_obstacle_in_a_batch(sph, gpu):
    """In a batch the obstacle applies to every scene in its own coordinates: after one step two
    identical scenes match each other and the same scene stepped alone with the obstacle up to
    FP32 rounding (a batch places row segments at other shared-memory offsets, so the packed
    density lanes differ; see test_batched_matches_single_scenes), and after six steps no
    particle of either scene is inside the sphere."""
    p = sph.workload_params(lower=(0.0, 0.0, 0.0), upper=(0.3, 0.3, 0.3))
    parts = sph.scene_fill(3000, (0.05, 0.05, 0.05), (0.25, 0.2, 0.25), 0.5 * p.h, 0.01 * p.h, 9)
    sdf = sphere_sdf(16, 0.02, (0.15, 0.1, 0.15), 0.05)
    n = len(parts)
    counts = np.array([n, n], dtype=np.uint32)

    def depth(x):
        return 0.05 - np.linalg.norm(x[:, :3].astype(np.float64) - (0.15, 0.1, 0.15), axis=1)

    assert (depth(parts["pos"]) > 0.0).sum() > 100  # the lattice starts partly inside
    with sph.Sim([p, p], counts=counts) as b, sph.Sim(p, n_max=n) as one:
        b.upload(np.concatenate([parts, parts]))
        one.upload(parts)
        for sim in (b, one):
            sim.set_obstacle(sdf, (0.0, 0.0, 0.0), 0.02)
            sim.step(1)
        out, ref = b.download(), one.download()
        for g in (out["pos"][:n], out["pos"][n:]):
            np.testing.assert_allclose(g[:, :3], ref["pos"][:, :3], rtol=0, atol=1e-6)
        b.step(5)
        out = b.download()
    for x in (out["pos"][:n], out["pos"][n:]):  # within the sampling error of a 0.02 grid on r = 0.05
        assert depth(x).max() < 5e-3
