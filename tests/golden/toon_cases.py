"""Seeded fragment cases for pinning the render restatement's shading to the reference's
toon_fs.glsl (celshading() in SPH mode, outline()): shared by tests/golden/make_golden.py,
which stores the reference shader's answers, and tests/test_render_pin.py, which checks the
restatement against them. numpy's PCG64 streams are the same on every platform."""
from __future__ import annotations

import itertools

import numpy as np

N_CEL = 20000
SHININESS = (0.3, 1.0, 5.0, 32.0)  # 0.3: the reference's default (Main.cpp:130)


def cel_cases(n: int = N_CEL, seed: int = 2024):
    """Per fragment: world position pw, eye and light positions, gl_PointCoord pc (FP32) and a
    shininess. Positions around a unit scene, the eye a few units away, the light anywhere."""
    rng = np.random.default_rng(seed)
    pw = rng.uniform(-1.0, 1.0, (n, 3)).astype(np.float32)
    eye = (rng.normal(0.0, 1.0, (n, 3)) * 3.0 + np.array([0.0, 1.0, 5.0])).astype(np.float32)
    light = rng.uniform(-6.0, 6.0, (n, 3)).astype(np.float32)
    pc = rng.uniform(0.0, 1.0, (n, 2)).astype(np.float32)
    shin = np.asarray(SHININESS, dtype=np.float32)[rng.integers(0, len(SHININESS), n)]
    return pw, eye, light, pc, shin


def outline_cases() -> np.ndarray:
    """Every 0/1 coverage pattern of a 3 x 3 neighbourhood: (512, 9), entry 3 i + j at (x + i - 1, y + j - 1)."""
    return np.array(list(itertools.product((0, 1), repeat=9)), dtype=np.int32)


def point_to_p(pc: np.ndarray) -> np.ndarray:
    """p = 2 gl_PointCoord - 1 in FP32, as toon_fs.glsl:97 computes it."""
    pc = np.asarray(pc, dtype=np.float32)
    return (np.float32(2.0) * pc - np.float32(1.0)).astype(np.float32)
