"""Benchmark scenes built on the CPU without the product library. TEST INFRASTRUCTURE ONLY.

The CPU legs of bench.py (the reference arm and the cpu_baseline) time the oracle on the
same seeded scenes the GPU path runs; this module builds them in numpy so that those legs
load nothing but oracle/. It restates:
  - sph_params (include/sph_gb300.h): the reference's ConstantsUniform and BoundaryUniform
    (NPR-SPH/Main.cpp:110-122) plus the shader constants (rho_pres_comp.glsl:3-8, :33,
    force_comp.glsl:33, integrate_comp.glsl:8, :33), as a ctypes structure of the same layout;
  - the seeded jittered lattice of sph_scene_fill (splitmix64 stream, the same double
    arithmetic, rounded once to float32), so that the scenes are identical byte for byte
    (tests/test_oracle_scenes.py pins that against the library);
  - the dam break and the 10,000-particle reference-box scene of the benchmark.
"""
from __future__ import annotations

import ctypes as C
import os
import platform

import numpy as np

PARTICLE_DTYPE = np.dtype([("pos", "<f4", 4), ("vel", "<f4", 4), ("force", "<f4", 4), ("extras", "<f4", 4)])


class Params(C.Structure):
    """sph_params of include/sph_gb300.h (ABI layout)."""

    _fields_ = [("mass", C.c_float), ("smoothing_coeff", C.c_float), ("visc", C.c_float),
                ("resting_rho", C.c_float), ("upper", C.c_float * 4), ("lower", C.c_float * 4),
                ("particle_radius", C.c_float), ("gas_const", C.c_float), ("gravity", C.c_float * 3),
                ("dt", C.c_float), ("damping", C.c_float), ("cell_scale", C.c_float), ("flags", C.c_uint32),
                ("reserved", C.c_uint32 * 3)]

    @property
    def h(self) -> float:
        return float(np.float32(self.smoothing_coeff) * np.float32(self.particle_radius))  # rho_pres_comp.glsl:40


def default_params() -> Params:
    """The reference's literal uniforms and shader constants."""
    p = Params()
    p.mass, p.smoothing_coeff, p.visc, p.resting_rho = 0.02, 4.0, 3000.0, 1000.0   # Main.cpp:112-115
    for a, (u, lo) in enumerate(zip((0.5, 1.0, 0.5, 1.0), (-0.1, -0.35, -0.1, 1.0))):  # Main.cpp:120-121
        p.upper[a], p.lower[a] = u, lo
    p.particle_radius = 0.005                                                       # rho_pres_comp.glsl:5
    p.gas_const = 2000.0                                                            # rho_pres_comp.glsl:33
    p.gravity[0], p.gravity[1], p.gravity[2] = 0.0, -9806.65, 0.0                   # force_comp.glsl:33
    p.dt = 1.0 / 10000                                                              # integrate_comp.glsl:33
    p.damping = 0.3                                                                 # integrate_comp.glsl:8
    return p


def workload_params(lower=None, upper=None) -> Params:
    """The benchmark scenes' uniforms: literal m, h, rho0, k, mu and damping with gravity
    (0, -9.81, 0) and a fixed dt of 1e-4."""
    p = default_params()
    p.gravity[1] = -9.81
    p.dt = 1e-4
    for a in range(3):
        if lower is not None:
            p.lower[a] = lower[a]
        if upper is not None:
            p.upper[a] = upper[a]
    return p


_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix(seed: int, ctr: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser of seed + (ctr + 1) * golden gamma (uint64 arithmetic wraps)."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + (ctr.astype(np.uint64) + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def scene_fill(n: int, lo, hi, spacing: float, jitter: float, seed: int) -> np.ndarray:
    """n records on the lattice of spacing `spacing` filling [lo, hi] (x fastest, then z, then
    y), each coordinate jittered by jitter * U[-1, 1) (24-bit uniform from the splitmix64
    stream at counter 3 idx + axis); pos.w = 1, everything else zero."""
    lo32 = np.asarray(lo, dtype=np.float32).astype(np.float64)
    hi32 = np.asarray(hi, dtype=np.float32).astype(np.float64)
    sp = float(np.float32(spacing))
    jt = float(np.float32(jitter))
    cnt = [int(np.floor((hi32[a] - lo32[a]) / sp + 1e-6)) if hi32[a] > lo32[a] else 0 for a in range(3)]
    if cnt[0] * cnt[1] * cnt[2] < n:
        raise ValueError("the lattice does not hold n particles")
    idx = np.arange(n, dtype=np.int64)
    ic = [idx % cnt[0], idx // (cnt[0] * cnt[2]), (idx // cnt[0]) % cnt[2]]  # x, y, z
    out = np.zeros(n, dtype=PARTICLE_DTYPE)
    for a in range(3):
        u = (_splitmix(seed, 3 * idx + a) >> np.uint64(40)).astype(np.float64) / float(1 << 23) - 1.0
        out["pos"][:, a] = (lo32[a] + (ic[a].astype(np.float64) + 0.5) * sp + jt * u).astype(np.float32)
    out["pos"][:, 3] = 1.0
    return out


def dam_break(nx: int = 64, ny: int = 128, nz: int = 128, seed: int = 2) -> tuple[Params, np.ndarray]:
    """The dam break of the benchmark: an nx*ny*nz block at 0.5h (jitter 0.01h) against the
    x = 0 wall of a 4:1:1 box whose y and z extents equal the block's."""
    h = default_params().h
    s = 0.5 * h
    bx, by, bz = nx * s, ny * s, nz * s
    L = max(by, bz)
    p = workload_params(lower=(0.0, 0.0, 0.0), upper=(4 * L, by, bz))
    parts = scene_fill(nx * ny * nz, (0.0, 0.0, 0.0), (bx, by, bz), s, 0.01 * p.h, seed)
    return p, parts


def reference_scene_10k(seed: int = 1) -> tuple[Params, np.ndarray]:
    """10,000 particles at 0.5h (jitter 0.01h) filling the lower-corner quarter of the
    reference box (half of x, half of z, from the floor up)."""
    p = workload_params()
    h = p.h
    lo = [p.lower[a] for a in range(3)]
    hi = [p.lower[0] + 0.5 * (p.upper[0] - p.lower[0]), p.upper[1], p.lower[2] + 0.5 * (p.upper[2] - p.lower[2])]
    return p, scene_fill(10000, lo, hi, 0.5 * h, 0.01 * h, seed)


def cpu_model() -> str:
    """The host CPU's model name (lscpu's on Arm, /proc/cpuinfo's on x86-64), with the
    machine type."""
    name = ""
    try:
        import subprocess

        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() in ("Model name", "Model"):
                name = line.split(":", 1)[1].strip()
                if line.startswith("Model name"):
                    break
    except (OSError, ValueError):
        pass
    if not name and os.path.exists("/proc/cpuinfo"):
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                name = line.split(":", 1)[1].strip()
                break
    return f"{name or 'unknown'} ({platform.machine()}, {os.cpu_count()} logical CPUs)"
