"""Generate tests/golden/reference_shader.npz from the reference's own compute shaders.

The three GLSL shaders of NPR-SPH (rho_pres_comp.glsl, force_comp.glsl,
integrate_comp.glsl) are compiled as C++ by `make -C oracle ref` (see
oracle/ref_shader/) and stepped on the CPU. This script needs the reference
tree and is run by hand where it is present, with $NPRSPH_REF_DIR naming its
NPR-SPH/ folder (the one holding the .glsl files):

    NPRSPH_REF_DIR=<reference>/NPR-SPH python tests/golden/make_golden.py

The fixture holds, per case and step count:
  - sha256 of the full 10,000-record output (bit-exact pin of the FP32 mirror),
  - every 20th record of the output (float32, for readable diffs),
  - sha256 of the input scene (pins the scene generator).
It also writes tests/golden/reference_toon.npz: the reference's particle fragment shader
(toon_fs.glsl, celshading() and outline()) on the seeded cases of toon_cases.py.

Cases (the shaders hard-code NUM_PARTICLES = 10000, G = -9806.65, k = 2000, dt = 1e-4):
  literal   make_grid() of Main.cpp:488-505 (10x100x10 at 0.005), the reference's own start
  lattice   10,000 points at 0.5h, jitter +-0.01h, seed 1, in the lower-corner quarter of the box
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
sys.path[:0] = [str(REPO / "npr-sph_gb300"), str(REPO)]

import nprsph as S  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent / "reference_shader.npz"
OUT_TOON = Path(__file__).resolve().parent / "reference_toon.npz"
STEPS = {"literal": (1, 3, 20), "lattice": (1, 3, 20)}
SUB = slice(0, None, 20)


def scenes():
    lit = S.scene_reference_grid()
    sc = S.reference_scene_10k(seed=1)
    return {"literal": lit, "lattice": sc.particles}


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main() -> None:
    O.build(with_ref=True)
    assert O.ref_available(), "oracle/_ref/libref_shader.so was not built (set NPRSPH_REF_DIR)"
    data = {}
    for name, parts in scenes().items():
        data[f"{name}_input_sha"] = np.array(sha(parts))
        for n in STEPS[name]:
            out = O.ref_shader_step(parts, n)
            data[f"{name}_s{n}_sha"] = np.array(sha(out))
            data[f"{name}_s{n}_sub"] = np.ascontiguousarray(out[SUB]).view(np.float32).reshape(-1, 16).copy()
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")
    toon()


def toon() -> None:
    """The reference's toon_fs.glsl (compiled as C++, oracle/_ref/libref_toon.so) on the seeded
    cases of toon_cases.py: celshading()'s choice per fragment (-1 discard, 0 dark, 1 midtone,
    2 highlight) and outline()'s decision per 3 x 3 coverage pattern."""
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    import toon_cases as TC

    assert O.ref_toon_available(), "oracle/_ref/libref_toon.so was not built (set NPRSPH_REF_DIR)"
    pw, eye, light, pc, shin = TC.cel_cases()
    cel = np.array([O.ref_toon_cel(pw[i], eye[i], light[i], pc[i], float(shin[i])) for i in range(len(pw))],
                   dtype=np.int8)
    cov = TC.outline_cases()
    outl = np.array([O.ref_toon_outline(c.astype(np.float32)) for c in cov], dtype=np.int8)
    inputs = hashlib.sha256(b"".join(np.ascontiguousarray(a).tobytes() for a in (pw, eye, light, pc, shin))).hexdigest()
    np.savez_compressed(OUT_TOON, cel=cel, outline=outl, inputs_sha=np.array(inputs))
    print(f"wrote {OUT_TOON} ({OUT_TOON.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
