"""Host-side checks of libsph_gb300.so that need no GPU: it loads, exports every function
declared in include/sph_gb300.h, and its parameter logic and scene generators behave."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

HEADER = Path(__file__).resolve().parents[1] / "include" / "sph_gb300.h"


def declared_functions() -> list[str]:
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(sph_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(sph):
    names = declared_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(sph.lib, n), n
    assert set(names) == set(sph._SIGS), set(names) ^ set(sph._SIGS)


def test_struct_layouts(sph):
    assert C.sizeof(sph.Params) == 96
    assert sph.PARTICLE_DTYPE.itemsize == 64
    assert sph.lib.sph_version().decode().startswith("sph_gb300")


def test_defaults_are_the_reference_literals(sph):
    p = sph.default_params()
    assert (p.mass, p.smoothing_coeff, p.visc, p.resting_rho) == pytest.approx((0.02, 4.0, 3000.0, 1000.0))
    assert list(p.upper) == pytest.approx([0.5, 1.0, 0.5, 1.0])
    assert list(p.lower) == pytest.approx([-0.1, -0.35, -0.1, 1.0])
    assert p.particle_radius == pytest.approx(0.005)
    assert p.gas_const == 2000.0
    assert list(p.gravity) == pytest.approx([0.0, -9806.65, 0.0])
    assert p.dt == np.float32(1.0) / np.float32(10000)
    assert p.damping == pytest.approx(0.3)
    assert p.h == float(np.float32(4.0) * np.float32(0.005))
    assert sph.lib.sph_params_validate(C.byref(p)) == 0


@pytest.mark.parametrize("field,value", [("mass", 0.0), ("resting_rho", -1.0), ("dt", 0.0),
                                         ("smoothing_coeff", float("nan")), ("visc", float("inf")),
                                         ("flags", 0x80), ("cell_scale", -1.0)])
def test_validate_rejects(sph, field, value):
    p = sph.default_params()
    setattr(p, field, value)
    assert sph.lib.sph_params_validate(C.byref(p)) == sph.ERR_INVALID_ARG


def test_validate_rejects_inverted_box_and_reserved(sph):
    p = sph.default_params()
    p.lower[1] = 2.0
    assert sph.lib.sph_params_validate(C.byref(p)) == sph.ERR_INVALID_ARG
    p = sph.default_params()
    p.reserved[1] = 3
    assert sph.lib.sph_params_validate(C.byref(p)) == sph.ERR_INVALID_ARG


def test_create_rejects_bad_arguments_before_any_cuda_call(sph):
    ctx = C.c_void_p()
    p = sph.default_params()
    p.mass = -1.0
    assert sph.lib.sph_create(C.byref(p), 100, None, C.byref(ctx)) == sph.ERR_INVALID_ARG
    p = sph.default_params()
    assert sph.lib.sph_create(C.byref(p), 0, None, C.byref(ctx)) == sph.ERR_INVALID_ARG
    assert sph.lib.sph_create(None, 10, None, C.byref(ctx)) == sph.ERR_INVALID_ARG
    counts = (C.c_uint32 * 2)(5, 0)
    plist = (sph.Params * 2)(p, p)
    assert sph.lib.sph_create_batch(plist, counts, 2, None, C.byref(ctx)) == sph.ERR_INVALID_ARG
    assert sph.lib.sph_step(None, 1) == sph.ERR_INVALID_ARG
    assert sph.lib.sph_destroy(None) == sph.ERR_INVALID_ARG


def test_grid_dims(sph):
    e, d = sph.grid_dims(sph.default_params())
    assert e == pytest.approx(0.02 * (1 + 1 / 1024), rel=1e-6)
    assert d == (30, 68, 30)
    db = sph.dam_break()
    e, d = sph.grid_dims(db.params)
    assert d == (256, 64, 64)


def test_reference_grid_layout(sph):
    a = sph.scene_reference_grid()
    i, j, k = 3, 57, 8
    idx = (i * 100 + j) * 10 + k  # Main.cpp:493-503 loop order
    np.testing.assert_array_equal(a["pos"][idx], np.float32([i * np.float32(0.005), j * np.float32(0.005),
                                                             k * np.float32(0.005), 1.0]))
    assert np.all(a["vel"] == 0) and np.all(a["force"] == 0) and np.all(a["extras"] == 0)


def test_fill_scene(sph):
    lo, hi, s = (0.0, 0.0, 0.0), (0.1, 0.2, 0.1), 0.01
    a = sph.scene_fill(500, lo, hi, s, 2e-4, 9)
    b = sph.scene_fill(500, lo, hi, s, 2e-4, 9)
    c = sph.scene_fill(500, lo, hi, s, 2e-4, 10)
    np.testing.assert_array_equal(a, b)
    assert not np.array_equal(a, c)
    z = sph.scene_fill(500, lo, hi, s, 0.0, 9)
    d = a["pos"][:, :3] - z["pos"][:, :3]
    assert np.abs(d).max() <= 2e-4 + 1e-7 and np.abs(d).max() > 1e-4
    # x fastest, then z, then y
    np.testing.assert_allclose(z["pos"][:3, :3], [[0.005, 0.005, 0.005], [0.015, 0.005, 0.005],
                                                  [0.025, 0.005, 0.005]], rtol=1e-6)
    np.testing.assert_allclose(z["pos"][10, :3], [0.005, 0.005, 0.015], rtol=1e-6)
    np.testing.assert_allclose(z["pos"][100, :3], [0.005, 0.015, 0.005], rtol=1e-6)
    with pytest.raises(sph.SphError):
        sph.scene_fill(5000, lo, hi, s, 0.0, 1)


def test_ball_scene(sph):
    a = sph.scene_ball(1000, (0.5, 0.5, 0.5), 0.01, 0.0, 1)
    r = np.linalg.norm(a["pos"][:, :3] - 0.5, axis=1)
    assert r.max() < 0.01 * (3 * 1000 / (4 * np.pi)) ** (1 / 3) + 0.02
    assert len(np.unique(a["pos"][:, :3], axis=0)) == 1000
    np.testing.assert_allclose(a["pos"][:, :3].mean(0), 0.5, atol=2e-3)


def test_benchmark_scenes(sph):
    s1 = sph.reference_scene_10k()
    assert len(s1.particles) == 10000
    p = s1.params
    pos = s1.particles["pos"][:, :3]
    assert np.all(pos >= np.array(p.lower[:3]) - 1e-6)
    assert pos[:, 0].max() < p.lower[0] + 0.5 * (p.upper[0] - p.lower[0])
    assert list(p.gravity) == pytest.approx([0.0, -9.81, 0.0])
    s2 = sph.dam_break(16, 32, 32)
    assert len(s2.particles) == 16 * 32 * 32
    plist, counts, parts = sph.batched_scenes(16, seed=3)
    assert len(plist) == 16 and len(parts) == counts.sum()
    assert counts.min() >= 2000 and counts.max() <= 65536
    for q in plist:
        assert 500 <= q.gas_const <= 3000 and 0.1 <= q.visc <= 2.0


def test_slosh_field(sph):
    s = sph.slosh_block(16)
    L = s.params.upper[0] - s.params.lower[0]
    x = s.particles["pos"][:, 0].astype(np.float64)
    np.testing.assert_allclose(s.particles["vel"][:, 0], 0.5 * np.sin(np.pi * x / L), atol=1e-6)
