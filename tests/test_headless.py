"""The C++ host loop (npr-sph_gb300/host/sph_headless.cpp): Main.cpp's frame loop over the C ABI
with scripted key presses ('p' pause/resume, starting paused; 'r' reset)."""
from __future__ import annotations

import json
import subprocess
from pathlib import Path

import pytest

BIN = Path(__file__).resolve().parents[1] / "npr-sph_gb300" / "sph_headless"


def run(*args, timeout=300):
    return subprocess.run([str(BIN), *args], capture_output=True, text=True, timeout=timeout)


def test_rejects_bad_arguments():
    assert BIN.exists()
    assert run("--bogus").returncode == 2
    assert run("--keys", "@3").returncode == 2
    assert run("--scene", "nope").returncode == 2


@pytest.mark.gpu
def test_scripted_frames(gpu):
    # frames 0-49: paused (the reference starts paused); p@50 -> 50 steps; r@100 resets the step
    # count; p@120 pauses; p@130 resumes -> 20 more steps by frame 150
    r = run("--frames", "150", "--keys", "p@50,r@100,p@120,p@130", "--report", "50")
    assert r.returncode == 0, r.stderr
    lines = [json.loads(x) for x in r.stdout.splitlines()]
    assert [x["frame"] for x in lines] == [50, 100, 150]
    assert [x["steps"] for x in lines] == [0, 50, 40]
    assert all(x["nonfinite"] == 0 for x in lines)
    assert lines[1]["mean_rho"] > 3900.0


@pytest.mark.gpu
def test_uniform_edits_take_effect(gpu):
    a = run("--frames", "40", "--keys", "p@0", "--report", "40")
    b = run("--frames", "40", "--keys", "p@0", "--report", "40", "--visc", "1000", "--rest-rho", "2000")
    assert a.returncode == 0 and b.returncode == 0, (a.stderr, b.stderr)
    ka = json.loads(a.stdout.splitlines()[-1])["kinetic_energy"]
    kb = json.loads(b.stdout.splitlines()[-1])["kinetic_energy"]
    assert ka != kb


@pytest.mark.gpu
def test_render_frames_to_ppm(gpu, tmp_path):
    prefix = tmp_path / "f"
    r = run("--frames", "40", "--keys", "p@0", "--report", "40", "--render-every", "20",
            "--render-prefix", str(prefix), "--size", "320x240")
    assert r.returncode == 0, r.stderr
    for k in (20, 40):
        data = (tmp_path / f"f_{k:05d}.ppm").read_bytes()
        assert data.startswith(b"P6\n320 240\n255\n")
        assert len(data) == len(b"P6\n320 240\n255\n") + 320 * 240 * 3


@pytest.mark.gpu
def test_obstacle_mesh(sph, gpu, tmp_path):
    """--obstacle: an icosphere OBJ through the reference's lattice becomes a static obstacle (the
    particles inside it are moved out in the first step); the run stays finite and its state
    differs from the same run without the mesh."""
    v, t = sph.icosphere(0.03, (0.02, 0.25, 0.02), 2)
    sph.write_obj(tmp_path / "ball.obj", v, t)
    a = run("--frames", "30", "--keys", "p@0", "--report", "30", "--obstacle", str(tmp_path / "ball.obj"))
    b = run("--frames", "30", "--keys", "p@0", "--report", "30")
    assert a.returncode == 0 and b.returncode == 0, (a.stderr, b.stderr)
    assert "320 triangles" in a.stderr
    la, lb = json.loads(a.stdout.splitlines()[-1]), json.loads(b.stdout.splitlines()[-1])
    assert la["nonfinite"] == 0 and la["steps"] == 30
    assert la["kinetic_energy"] != lb["kinetic_energy"]
    assert run("--obstacle", str(tmp_path / "missing.obj"), "--frames", "1").returncode == 1
