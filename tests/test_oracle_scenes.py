"""The oracle's numpy scene builders (used by bench.py's CPU legs, which load nothing of the
product) give the library's scenes byte for byte: parameters and particle records."""
from __future__ import annotations

import ctypes as C

import pytest


@pytest.mark.parametrize("shape,seed", [((64, 128, 128), 2), ((32, 64, 64), 2), ((16, 32, 32), 3), ((8, 8, 8), 11)])
def test_dam_break_matches_library(sph, shape, seed):
    from oracle import scenes as OS

    lib = sph.dam_break(*shape, seed=seed)
    p, parts = OS.dam_break(*shape, seed=seed)
    assert C.sizeof(p) == C.sizeof(lib.params) == 96
    assert bytes(p) == bytes(lib.params)
    assert parts.dtype.itemsize == 64
    assert parts.tobytes() == lib.particles.tobytes()


def test_reference_scene_matches_library(sph):
    from oracle import scenes as OS

    lib = sph.reference_scene_10k(seed=1)
    p, parts = OS.reference_scene_10k(seed=1)
    assert bytes(p) == bytes(lib.params)
    assert parts.tobytes() == lib.particles.tobytes()


def test_default_params_match_library(sph):
    from oracle import scenes as OS

    assert bytes(OS.default_params()) == bytes(sph.default_params())


def test_cpu_model_names_the_machine():
    from oracle import scenes as OS

    s = OS.cpu_model()
    assert "logical CPUs" in s and len(s) > 10
