"""The render restatement (oracle/render_oracle.cpp, the CPU check of sph_render) pinned to the
reference's own particle fragment shader, NPR-SPH/toon_fs.glsl, compiled as C++
(oracle/ref_shader/ref_toon.cpp): celshading() in SPH mode (toon_fs.glsl:90-124) and outline()
(:126-153), including its `g > 0.1` threshold. The shader's answers on seeded cases are
committed in tests/golden/reference_toon.npz (tests/golden/make_golden.py made them); where the
reference tree was present at build time they are also recomputed live.

The restatement tests `r.v > 0 and r.v > 0.95^(1/shininess)` where the shader tests
`pow(r.v, shininess) > 0.95`: equal in exact arithmetic (pow of a negative r.v is undefined in
GLSL and NaN on GPUs, exp2(y log2 x), for a uniform exponent; the C++ build of the shader follows
that, and expands the literal pow(g, 2.0) of outline() into g * g as GPU compilers do), and in
FP32 they may differ only for fragments with pow(r.v, shininess) within PIN_BAND of 0.95."""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))
import toon_cases as TC  # noqa: E402

PIN_BAND = 1e-5


def thr_of(s: float) -> float:
    """0.95^(1/shininess) as the restatement forms it (FP64, rounded once)."""
    return float(np.float32(0.95 ** (1.0 / float(s))))


@pytest.fixture(scope="module")
def golden():
    d = np.load(GOLDEN / "reference_toon.npz")
    pw, eye, light, pc, shin = TC.cel_cases()
    sha = hashlib.sha256(b"".join(np.ascontiguousarray(a).tobytes() for a in (pw, eye, light, pc, shin))).hexdigest()
    assert sha == str(d["inputs_sha"]), "the seeded cases changed"
    return d


def test_outline_matches_reference_shader(orc, golden):
    cov = TC.outline_cases()
    ours = np.array([orc.toon_outline(c) for c in cov])
    np.testing.assert_array_equal(ours, golden["outline"])
    # the threshold: with 0/1 coverage the gradient is 0 or at least 1, so g > 0.1 means g != 0
    assert golden["outline"].sum() == 464 and int((golden["outline"] == 0).sum()) == 48


def test_cel_shading_matches_reference_shader(orc, golden):
    pw, eye, light, pc, shin = TC.cel_cases()
    p = TC.point_to_p(pc)
    ref = golden["cel"].astype(int)
    ours = np.zeros(len(pw), int)
    rvs = np.zeros(len(pw), np.float32)
    for i in range(len(pw)):
        ours[i], rvs[i] = orc.toon_cel(pw[i], eye[i], light[i], float(p[i, 0]), float(p[i, 1]), thr_of(shin[i]))
    assert np.array_equal(ours == -1, ref == -1), "discard decisions differ"
    with np.errstate(invalid="ignore"):
        pv = np.power(rvs.astype(np.float32), shin.astype(np.float32)).astype(np.float64)
    near = np.abs(pv - 0.95) <= PIN_BAND
    diff = ours != ref
    assert not np.any(diff & ~near), np.flatnonzero(diff & ~near)[:10]
    assert diff.sum() <= 5, diff.sum()
    assert set(np.unique(ref)) == {-1, 0, 1, 2}  # every outcome occurs in the cases


def test_live_reference_shader_reproduces_golden(orc, golden):
    if not orc.ref_toon_available():
        pytest.skip("oracle/_ref/libref_toon.so not built (no reference tree at build time)")
    pw, eye, light, pc, shin = TC.cel_cases()
    live = np.array([orc.ref_toon_cel(pw[i], eye[i], light[i], pc[i], float(shin[i])) for i in range(2000)])
    np.testing.assert_array_equal(live, golden["cel"][:2000])
    cov = TC.outline_cases()
    live_o = np.array([orc.ref_toon_outline(c.astype(np.float32)) for c in cov])
    np.testing.assert_array_equal(live_o, golden["outline"])
