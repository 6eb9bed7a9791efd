"""Headless toon rendering (sph_render) of the reference's SPH-mode draw: the view matrices
against a numpy restatement of the glm formulas, the CPU oracle (oracle/render_oracle.cpp) on
known answers, and the CUDA image byte for byte against the oracle."""
from __future__ import annotations

import math

import numpy as np
import pytest


def glm_like(angle, scale, eye, center, aspect):
    """rotate(angle, y) * scale, lookAt(eye, center, y), perspective(pi/4, aspect, 0.1, 100) as
    row-major numpy matrices (Main.cpp:256-258)."""
    c, s = math.cos(angle), math.sin(angle)
    M = np.array([[c, 0, s, 0], [0, 1, 0, 0], [-s, 0, c, 0], [0, 0, 0, 1]]) @ np.diag([scale, scale, scale, 1])
    f = np.asarray(center, float) - np.asarray(eye, float)
    f /= np.linalg.norm(f)
    r = np.cross(f, [0, 1, 0])
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    V = np.eye(4)
    V[0, :3], V[1, :3], V[2, :3] = r, u, -f
    V[:3, 3] = [-r @ eye, -u @ eye, f @ eye]
    t = math.tan(math.pi / 8)
    P = np.zeros((4, 4))
    P[0, 0], P[1, 1] = 1 / (aspect * t), 1 / t
    P[2, 2], P[2, 3], P[3, 2] = -(100.1) / 99.9, -(2 * 100 * 0.1) / 99.9, -1.0
    return M, V, P


def as_rowmajor(a) -> np.ndarray:
    return np.array(a[:], dtype=np.float64).reshape(4, 4).T  # column-major storage


def test_view_default_matches_glm_formulas(sph):
    v = sph.view_default(800, 600, 1.0)
    M, V, P = glm_like(0.75, 2.5, [10.0, 2.0, 0.0], [0.0, 0.0, 0.0], 800 / 600)
    for got, ref in ((v.model, M), (v.view, V), (v.proj, P)):
        np.testing.assert_allclose(as_rowmajor(got), ref, rtol=0, atol=1e-6)
    assert list(v.light_w) == [0.0, 1.0, 1.0, 1.0] and v.point_size == 10.0
    assert abs(v.shininess - 0.3) < 1e-7 and list(v.clear_color[:3]) == [0.5, 0.5, 0.5]


def test_oracle_single_particle_disc_and_outline(sph, orc):
    v = sph.view_default(64, 48, 1.0)
    v.clear_color[:3] = [0.2, 0.4, 0.6]  # the default clear grey equals the midtone
    img = orc.render(v, np.array([[0.0, 0.0, 0.0, 1.0]], np.float32))  # projects to the image centre
    clear = np.array([51, 102, 153, 255], np.uint8)
    cov = np.any(img != clear, axis=-1)
    xs = np.arange(64) + 0.5 - 32.0
    ys = np.arange(48) + 0.5 - 24.0
    px, py = np.meshgrid(xs / 5.0, ys / 5.0)
    box = (np.abs(xs)[None, :] <= 5.0) & (np.abs(ys)[:, None] <= 5.0) & (xs[None, :] < 5.0) & (ys[:, None] < 5.0)
    expect = box & (px * px + py * py <= 1.0)
    assert np.array_equal(cov, expect)
    # outline = covered pixels with an uncovered 8-neighbour whose Sobel gradient is non-zero
    pad = np.pad(expect.astype(int), 1)
    gx = (pad[:-2, :-2] + 2 * pad[1:-1, :-2] + pad[2:, :-2]) - (pad[:-2, 2:] + 2 * pad[1:-1, 2:] + pad[2:, 2:])
    gy = (pad[:-2, :-2] + 2 * pad[:-2, 1:-1] + pad[:-2, 2:]) - (pad[2:, :-2] + 2 * pad[2:, 1:-1] + pad[2:, 2:])
    ring = expect & ((gx != 0) | (gy != 0))
    black = np.all(img == np.array([0, 0, 0, 255], np.uint8), axis=-1)
    assert np.all(black[ring])
    inner = expect & ~ring
    assert inner.sum() > 0
    assert np.all(np.isin(img[inner][:, 0], [0, 128, 255]))


def test_oracle_depth_test_ignores_draw_order(sph, orc):
    v = sph.view_default(96, 96, 1.0)
    near = [0.3, 0.0, 0.02, 1.0]   # toward the eye at (10, 2, 0) after the model rotation
    far = [-0.3, 0.0, -0.02, 1.0]
    a = orc.render(v, np.array([near, far], np.float32))
    b = orc.render(v, np.array([far, near], np.float32))
    assert np.array_equal(a, b)
    c = orc.render(v, np.array([near, near], np.float32))  # equal depth: the first drawn stays
    d = orc.render(v, np.array([near], np.float32))
    assert np.array_equal(c, d)


def test_ppm_writer(sph, tmp_path):
    rgba = np.zeros((3, 4, 4), np.uint8)
    rgba[0, :, 0] = 255  # bottom row red
    rgba[2, :, 2] = 255  # top row blue
    path = tmp_path / "x.ppm"
    sph.write_ppm(path, rgba)
    data = path.read_bytes()
    assert data.startswith(b"P6\n4 3\n255\n")
    px = np.frombuffer(data[len(b"P6\n4 3\n255\n"):], np.uint8).reshape(3, 4, 3)
    assert np.all(px[0, :, 2] == 255) and np.all(px[2, :, 0] == 255)  # file rows top to bottom


def wide_view(sph, w, h, eye, center=(0.0, 0.0, 0.0), angle=0.0, size=6.0):
    v = sph.view_default(w, h, 1.0)
    sph.view_camera(v, angle, 1.0, eye, center)
    v.point_size = size
    return v


@pytest.mark.gpu
def test_render_matches_oracle_reference_scene(sph, orc, gpu):
    sc = sph.reference_scene_10k()
    with sph.Sim(sc.params, n_max=len(sc.particles)) as sim:
        sim.upload(sc.particles)
        sim.step(60)
        state = sim.download()
        v = sph.view_default(720, 720, 1.0)
        img = sim.render(v)
        v2 = wide_view(sph, 640, 480, (1.2, 0.6, 1.5), (0.2, 0.2, 0.2), size=12.0)
        img2 = sim.render(v2)
    assert np.any(img != img[0, 0])
    assert np.array_equal(img, orc.render(v, state["pos"]))
    assert np.array_equal(img2, orc.render(v2, state["pos"]))


@pytest.mark.gpu
def test_render_matches_oracle_dam_break_1m(sph, orc, gpu):
    sc = sph.dam_break(seed=2)
    with sph.Sim(sc.params, n_max=len(sc.particles)) as sim:
        sim.upload(sc.particles)
        sim.step(200)
        state = sim.download()
        v = wide_view(sph, 1280, 720, (2.56, 2.5, 6.0), (2.56, 0.5, 0.64), size=4.0)
        img = sim.render(v)
    cov = np.any(img != img[0, 0], axis=-1).mean()
    assert 0.02 < cov < 0.98
    assert np.array_equal(img, orc.render(v, state["pos"]))


@pytest.mark.gpu
def test_render_device_buffer_and_batch_scene(sph, orc, gpu):
    import torch

    plist, counts, parts = sph.batched_scenes(4, seed=8, n_lo=2000, n_hi=5000)
    with sph.Sim(plist, counts=counts) as sim:
        sim.upload(parts)
        sim.step(10)
        state = sim.download()
        first = int(np.sum(counts[:2]))
        pos = state["pos"][first:first + counts[2]]
        edge = float(plist[2].upper[0])
        v = wide_view(sph, 320, 240, (edge * 2.2, edge * 1.5, edge * 2.5), (edge / 2, edge / 3, edge / 2))
        host = sim.render(v, scene=2)
        dev = torch.zeros(240 * 320 * 4, dtype=torch.uint8, device="cuda")
        sim.render_device(v, dev.data_ptr(), scene=2)
        torch.cuda.synchronize()
    assert np.array_equal(dev.cpu().numpy().reshape(240, 320, 4), host)
    assert np.array_equal(host, orc.render(v, pos))
