"""ctypes wrapper of the CPU oracle. TEST INFRASTRUCTURE ONLY.

Only tests/, the smoke check of __graft_entry__ and the CPU legs of bench.py
may import this module. It loads
  oracle/liboracle.so          FP64 / FP32 restatement of the reference SPH step (sph_oracle.cpp)
  oracle/_ref/libref_shader.so the reference's GLSL compute shaders compiled as C++ (optional:
                               only where the reference tree was present at build time)
and `build()` compiles them with make.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libref_shader.so"
REF_TOON_LIB = HERE / "_ref" / "libref_toon.so"
# The reference tree (its NPR-SPH/ folder with the .glsl shaders), named by the environment;
# without it the reference shaders are not built.
REF_ENV = "NPRSPH_REF_DIR"

_P = C.c_void_p
_I64 = C.c_int64


def ref_source() -> Path | None:
    """The reference's NPR-SPH/ folder named by $NPRSPH_REF_DIR, if it holds the shaders."""
    d = os.environ.get(REF_ENV)
    if not d:
        return None
    p = Path(d)
    return p if (p / "rho_pres_comp.glsl").is_file() else None


def build(with_ref: bool = True) -> None:
    """Always a full rebuild (a few seconds): the tree moves between x86-64 and aarch64 hosts,
    and a library left from the other architecture must never be loaded. The reference
    shaders are built only when $NPRSPH_REF_DIR names the reference's NPR-SPH/ folder."""
    subprocess.run(["make", "-s", "-B", "-C", str(HERE)], check=True)
    src = ref_source() if with_ref else None
    if src is not None:
        subprocess.run(["make", "-s", "-B", "-C", str(HERE), "ref", f"REF_DIR={src}"], check=True)


_lib = None
_ref = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build(with_ref=False)
        L = C.CDLL(str(LIB))
        L.oracle_step_f64.restype = C.c_int
        L.oracle_step_f64.argtypes = [_P, _I64, _P, _P, C.c_int, C.c_int, _P, _P, _P, _P, _P, _P, _P]
        L.oracle_force_f64.restype = C.c_int
        L.oracle_force_f64.argtypes = [_P, _I64, _P, _P, _P, _P, C.c_int, C.c_int, _P, _P, _P, _P, _P]
        L.oracle_force_cond_f64.restype = C.c_int
        L.oracle_force_cond_f64.argtypes = [_P, _I64, _P, _P, _P, _P, C.c_int, C.c_int, _P]
        L.oracle_run_f64.restype = C.c_int
        L.oracle_run_f64.argtypes = [_P, _I64, _P, _P, _P, _P, C.c_int, C.c_int, C.c_int]
        L.oracle_step_f32_aos.restype = C.c_int
        L.oracle_step_f32_aos.argtypes = [_P, _P, _I64, C.c_int, C.c_int, C.c_int, C.c_int]
        L.oracle_neighbors.restype = C.c_int
        L.oracle_neighbors.argtypes = [_P, _I64, _P, _I64, _P, C.c_int, C.c_int, _P, _P]
        L.oracle_obstacle_f64.restype = C.c_int
        L.oracle_obstacle_f64.argtypes = [_P, _P, _P, _P, C.c_double, _I64, _P, _P, _P]
        L.oracle_neighbor_lists.restype = C.c_int64
        L.oracle_neighbor_lists.argtypes = [_P, _I64, _P, C.c_int, _P, _P, _I64]
        L.oracle_cutoff_d2.restype = C.c_float
        L.oracle_cutoff_d2.argtypes = [C.c_float]
        L.oracle_mix64.restype = C.c_uint64
        L.oracle_mix64.argtypes = [C.c_uint64]
        L.oracle_max_threads.restype = C.c_int
        L.oracle_render.restype = C.c_int
        L.oracle_render.argtypes = [_P, _P, _I64, _P]
        L.oracle_toon_cel.restype = C.c_int
        L.oracle_toon_cel.argtypes = [_P, _P, _P, C.c_float, C.c_float, C.c_float, _P]
        L.oracle_toon_outline.restype = C.c_int
        L.oracle_toon_outline.argtypes = [_P]
        _lib = L
    return _lib


def ref_available() -> bool:
    return REF_LIB.exists()


_toon = None


def ref_toon_available() -> bool:
    return REF_TOON_LIB.exists()


def ref_toon() -> C.CDLL:
    """The reference's toon_fs.glsl compiled as C++ (oracle/_ref/libref_toon.so)."""
    global _toon
    if _toon is None:
        T = C.CDLL(str(REF_TOON_LIB))
        T.ref_toon_cel.restype = C.c_int
        T.ref_toon_cel.argtypes = [_P, _P, _P, _P, C.c_float]
        T.ref_toon_outline.restype = C.c_int
        T.ref_toon_outline.argtypes = [_P, C.c_int, C.c_int]
        _toon = T
    return _toon


def _f32p(a) -> int:
    return np.ascontiguousarray(a, dtype=np.float32).ctypes.data


def toon_cel(pw, eye, light, px: float, py: float, thr: float) -> tuple[int, float]:
    """The render restatement's cel-shading choice of one fragment (-1 discard, 0 dark,
    1 midtone, 2 highlight) and its r.v."""
    a, b, c = (np.ascontiguousarray(x, dtype=np.float32) for x in (pw, eye, light))
    rv = C.c_float()
    k = lib().oracle_toon_cel(a.ctypes.data, b.ctypes.data, c.ctypes.data, px, py, thr, C.byref(rv))
    return int(k), float(rv.value)


def toon_outline(cov) -> int:
    c = np.ascontiguousarray(cov, dtype=np.int32).reshape(9)
    return int(lib().oracle_toon_outline(c.ctypes.data))


def ref_toon_cel(pw, eye, light, pc, shininess: float) -> int:
    """celshading() of the reference shader for one fragment (gl_PointCoord pc)."""
    a, b, c, d = (np.ascontiguousarray(x, dtype=np.float32) for x in (pw, eye, light, pc))
    return int(ref_toon().ref_toon_cel(a.ctypes.data, b.ctypes.data, c.ctypes.data, d.ctypes.data, shininess))


def ref_toon_outline(green, x: int = 5, y: int = 7) -> int:
    g = np.ascontiguousarray(green, dtype=np.float32).reshape(9)
    return int(ref_toon().ref_toon_outline(g.ctypes.data, x, y))


def ref() -> C.CDLL:
    global _ref
    if _ref is None:
        R = C.CDLL(str(REF_LIB))
        R.ref_shader_step.restype = C.c_int
        R.ref_shader_step.argtypes = [_P, C.c_int, _P, _P, _P, C.c_int]
        R.ref_shader_num_particles.restype = C.c_int
        _ref = R
    return _ref


BACKENDS = {"brute": 0, "grid": 1}


def _pp(params) -> int:
    return C.addressof(params)


def step_f64(params, particles: np.ndarray, backend: str = "grid", nthreads: int = 0) -> dict:
    """One FP64 step from the state of `particles` (64-byte records). Returns the density,
    pressure, force, force scale, new position/velocity and wall margin per particle."""
    n = len(particles)
    pos = np.ascontiguousarray(particles["pos"][:, :3], dtype=np.float64)
    vel = np.ascontiguousarray(particles["vel"][:, :3], dtype=np.float64)
    out = {k: np.zeros(n) for k in ("rho", "pres", "fscale", "margin")}
    for k in ("force", "pos", "vel"):
        out[k] = np.zeros((n, 3))
    rc = lib().oracle_step_f64(_pp(params), n, pos.ctypes.data, vel.ctypes.data, BACKENDS[backend], nthreads,
                               out["rho"].ctypes.data, out["pres"].ctypes.data, out["force"].ctypes.data,
                               out["fscale"].ctypes.data, out["pos"].ctypes.data, out["vel"].ctypes.data,
                               out["margin"].ctypes.data)
    assert rc == 0
    return out


def force_f64(params, particles: np.ndarray, rho, pres, backend: str = "grid", nthreads: int = 0) -> dict:
    """The force and integrate passes in FP64 from the state of `particles` and the given
    densities/pressures (so a GPU force pass is checked on the very inputs it consumed)."""
    n = len(particles)
    pos = np.ascontiguousarray(particles["pos"][:, :3], dtype=np.float64)
    vel = np.ascontiguousarray(particles["vel"][:, :3], dtype=np.float64)
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    pres = np.ascontiguousarray(pres, dtype=np.float64)
    out = {"rho": rho, "pres": pres, "fscale": np.zeros(n), "margin": np.zeros(n)}
    for k in ("force", "pos", "vel"):
        out[k] = np.zeros((n, 3))
    rc = lib().oracle_force_f64(_pp(params), n, pos.ctypes.data, vel.ctypes.data, rho.ctypes.data,
                                pres.ctypes.data, BACKENDS[backend], nthreads, out["force"].ctypes.data,
                                out["fscale"].ctypes.data, out["pos"].ctypes.data, out["vel"].ctypes.data,
                                out["margin"].ctypes.data)
    assert rc == 0
    cond = np.zeros(n)
    rc = lib().oracle_force_cond_f64(_pp(params), n, pos.ctypes.data, vel.ctypes.data, rho.ctypes.data,
                                     pres.ctypes.data, BACKENDS[backend], nthreads, cond.ctypes.data)
    assert rc == 0
    out["fcond"] = cond
    return out


def run_f64(params, pos: np.ndarray, vel: np.ndarray, n_steps: int, backend: str = "grid",
            nthreads: int = 0) -> tuple[np.ndarray, np.ndarray]:
    """n_steps FP64 steps in place on (n,3) float64 arrays. Returns (rho, pres) of the last step."""
    n = len(pos)
    assert pos.dtype == np.float64 and vel.dtype == np.float64 and pos.flags.c_contiguous
    rho, pres = np.zeros(n), np.zeros(n)
    rc = lib().oracle_run_f64(_pp(params), n, pos.ctypes.data, vel.ctypes.data, rho.ctypes.data,
                              pres.ctypes.data, n_steps, BACKENDS[backend], nthreads)
    assert rc == 0
    return rho, pres


def step_f32(params, particles: np.ndarray, n_steps: int = 1, backend: str = "brute", literal_nan: bool = False,
             nthreads: int = 0) -> np.ndarray:
    """FP32 literal mirror of the three shaders, n_steps steps on a copy of `particles`."""
    a = np.ascontiguousarray(particles).copy()
    rc = lib().oracle_step_f32_aos(_pp(params), a.ctypes.data, len(a), n_steps, BACKENDS[backend], nthreads,
                                   1 if literal_nan else 0)
    assert rc == 0
    return a


def neighbors(params, particles: np.ndarray, queries, backend: str = "grid", nthreads: int = 0):
    pos4 = np.ascontiguousarray(particles["pos"], dtype=np.float32)
    q = np.ascontiguousarray(queries, dtype=np.int64)
    cnt = np.zeros(len(q), dtype=np.uint32)
    dig = np.zeros(len(q), dtype=np.uint64)
    rc = lib().oracle_neighbors(_pp(params), len(pos4), pos4.ctypes.data, len(q), q.ctypes.data, BACKENDS[backend],
                                nthreads, cnt.ctypes.data, dig.ctypes.data)
    assert rc == 0
    return cnt, dig


def neighbor_lists(params, particles: np.ndarray, backend: str = "grid", cap: int = 1 << 24):
    pos4 = np.ascontiguousarray(particles["pos"], dtype=np.float32)
    n = len(pos4)
    off = np.zeros(n + 1, dtype=np.int64)
    items = np.zeros(cap, dtype=np.int64)
    tot = lib().oracle_neighbor_lists(_pp(params), n, pos4.ctypes.data, BACKENDS[backend], off.ctypes.data,
                                      items.ctypes.data, cap)
    assert tot <= cap
    return off, items[:tot]


def cutoff_d2(h: float) -> float:
    return float(lib().oracle_cutoff_d2(h))


def mix64(j: int) -> int:
    return int(lib().oracle_mix64(j))


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def ref_shader_step(particles: np.ndarray, n_steps: int, constants=(0.02, 4.0, 3000.0, 1000.0),
                    upper=(0.5, 1.0, 0.5, 1.0), lower=(-0.1, -0.35, -0.1, 1.0), nthreads: int = 0) -> np.ndarray:
    """The reference shaders themselves (compiled as C++) on a copy of 10,000 records."""
    R = ref()
    assert len(particles) == R.ref_shader_num_particles()
    a = np.ascontiguousarray(particles).copy()
    c = (C.c_float * 4)(*constants)
    u = (C.c_float * 4)(*upper)
    lo = (C.c_float * 4)(*lower)
    rc = R.ref_shader_step(a.ctypes.data, n_steps, c, u, lo, nthreads)
    assert rc == 0
    return a


def render(view, pos4: np.ndarray) -> np.ndarray:
    """CPU restatement of the particle draw (render_oracle.cpp): `view` is an sph_view
    ctypes structure, pos4 the (n, 4) positions in record (draw) order. Returns the
    (height, width, 4) RGBA8 image, rows bottom to top."""
    pos4 = np.ascontiguousarray(pos4, dtype=np.float32)
    out = np.zeros((view.height, view.width, 4), dtype=np.uint8)
    rc = lib().oracle_render(C.addressof(view), pos4.ctypes.data, len(pos4), out.ctypes.data)
    assert rc == 0
    return out


def obstacle_f64(params, sdf: np.ndarray, origin, spacing: float, pos: np.ndarray, vel: np.ndarray):
    """The obstacle rule (FP64) on copies of pos/vel (n x 3) that already went through the wall
    clamp; sdf[z, y, x] as given to sph_set_obstacle. Returns (pos, vel, phi at the input)."""
    a = np.ascontiguousarray(sdf, dtype=np.float32)
    dims = np.array([a.shape[2], a.shape[1], a.shape[0]], dtype=np.int32)
    org = np.ascontiguousarray(origin, dtype=np.float64)
    x = np.array(pos, dtype=np.float64, order="C")
    v = np.array(vel, dtype=np.float64, order="C")
    phi = np.zeros(len(x))
    rc = lib().oracle_obstacle_f64(_pp(params), a.ctypes.data, dims.ctypes.data, org.ctypes.data, float(spacing),
                                   len(x), x.ctypes.data, v.ctypes.data, phi.ctypes.data)
    assert rc == 0
    return x, v, phi


def _tri_dist2(p: np.ndarray, a: np.ndarray, b: np.ndarray, c: np.ndarray) -> np.ndarray:
    """Squared distance from points p (m x 3) to triangle (a, b, c): the closest point by Voronoi
    region (Ericson, Real-Time Collision Detection, 2005, section 5.1.5), vectorised over p."""
    ab, ac = b - a, c - a
    ap, bp, cp = p - a, p - b, p - c
    d1, d2 = ap @ ab, ap @ ac
    d3, d4 = bp @ ab, bp @ ac
    d5, d6 = cp @ ab, cp @ ac
    va, vb, vc = d3 * d6 - d5 * d4, d5 * d2 - d1 * d6, d1 * d4 - d3 * d2
    with np.errstate(divide="ignore", invalid="ignore"):
        den = va + vb + vc
        q = a + np.outer(vb / den, ab) + np.outer(vc / den, ac)                              # face
        e_bc = (va <= 0) & (d4 - d3 >= 0) & (d5 - d6 >= 0)
        q = np.where(e_bc[:, None], b + np.outer((d4 - d3) / ((d4 - d3) + (d5 - d6)), c - b), q)
        e_ac = (vb <= 0) & (d2 >= 0) & (d6 <= 0)
        q = np.where(e_ac[:, None], a + np.outer(d2 / (d2 - d6), ac), q)
        v_c = (d6 >= 0) & (d5 <= d6)
        q = np.where(v_c[:, None], c, q)
        e_ab = (vc <= 0) & (d1 >= 0) & (d3 <= 0)
        q = np.where(e_ab[:, None], a + np.outer(d1 / (d1 - d3), ab), q)
        v_b = (d3 >= 0) & (d4 <= d3)
        q = np.where(v_b[:, None], b, q)
        v_a = (d1 <= 0) & (d2 <= 0)
        q = np.where(v_a[:, None], a, q)
    d = p - q
    return np.einsum("ij,ij->i", d, d)


def mesh_sdf(verts: np.ndarray, tris: np.ndarray, points: np.ndarray) -> np.ndarray:
    """FP64 signed distance of points (m x 3) to a closed triangle mesh: the distance to the
    nearest triangle, negative where the winding number (sum of solid angles by Van Oosterom
    and Strackee's formula, over 4 pi) exceeds 1/2. The restatement of sph_sdf_from_mesh."""
    v = np.asarray(verts, dtype=np.float64)
    p = np.asarray(points, dtype=np.float64)
    best = np.full(len(p), np.inf)
    omega = np.zeros(len(p))
    for ia, ib, ic in np.asarray(tris, dtype=np.int64):
        a, b, c = v[ia], v[ib], v[ic]
        best = np.minimum(best, _tri_dist2(p, a, b, c))
        x, y, z = a - p, b - p, c - p
        lx, ly, lz = (np.linalg.norm(t, axis=1) for t in (x, y, z))
        num = np.einsum("ij,ij->i", x, np.cross(y, z))
        den = lx * ly * lz + np.einsum("ij,ij->i", x, y) * lz + np.einsum("ij,ij->i", x, z) * ly + \
            np.einsum("ij,ij->i", y, z) * lx
        omega += 2.0 * np.arctan2(num, den)
    d = np.sqrt(best)
    return np.where(omega / (4.0 * np.pi) > 0.5, -d, d)
