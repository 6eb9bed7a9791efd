"""Python host binding of libsph_gb300.so (ctypes over the C ABI in include/sph_gb300.h).

It mirrors the reference host loop's view of the SPH step (NPR-SPH/Main.cpp):
the particle array (`struct Particle`, Main.cpp:93-99) is a numpy structured
array PARTICLE_DTYPE, the uniforms (Main.cpp:110-122 plus the shader constants)
are `Params`, and `Sim.step(n)` replaces the three dispatches of
Main.cpp:291-304. There is no fallback: if the library is missing or was not
built, importing this module raises.

The scene helpers build the seeded synthetic scenes of the benchmark
configurations (reference scene, dam break, batched boxes, slosh).
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("SPH_GB300_LIB", _HERE / "libsph_gb300.so"))

PARTICLE_DTYPE = np.dtype([("pos", "<f4", 4), ("vel", "<f4", 4), ("force", "<f4", 4), ("extras", "<f4", 4)])
assert PARTICLE_DTYPE.itemsize == 64

FLAG_KEEP_FORCE = 0x1
JUDGE_MEAN_DENSITY, JUDGE_PARTICLE_DENSITY = 0, 1
RECORDS_AUTO, RECORDS_ALWAYS, RECORDS_NEVER = 0, 1, 2

OK, ERR_INVALID_ARG, ERR_CUDA, ERR_OUT_OF_MEMORY, ERR_CAPACITY, ERR_NOT_READY, ERR_DEVICE, ERR_UNSUPPORTED = (
    0, -1, -2, -3, -4, -5, -6, -7)


class Params(C.Structure):
    """sph_params: ConstantsUniform + BoundaryUniform + shader constants (see include/sph_gb300.h)."""

    _fields_ = [("mass", C.c_float), ("smoothing_coeff", C.c_float), ("visc", C.c_float),
                ("resting_rho", C.c_float), ("upper", C.c_float * 4), ("lower", C.c_float * 4),
                ("particle_radius", C.c_float), ("gas_const", C.c_float), ("gravity", C.c_float * 3),
                ("dt", C.c_float), ("damping", C.c_float), ("cell_scale", C.c_float), ("flags", C.c_uint32),
                ("reserved", C.c_uint32 * 3)]

    @property
    def h(self) -> float:
        return float(np.float32(self.smoothing_coeff) * np.float32(self.particle_radius))

    def copy(self) -> "Params":
        p = Params()
        C.memmove(C.byref(p), C.byref(self), C.sizeof(Params))
        return p


class Diag(C.Structure):
    _fields_ = [("momentum", C.c_double * 3), ("kinetic_energy", C.c_double), ("potential_energy", C.c_double),
                ("mean_rho", C.c_double), ("min_rho", C.c_double), ("max_rho", C.c_double),
                ("mean_abs_rho_dev", C.c_double), ("nonfinite", C.c_uint64), ("n", C.c_uint64),
                ("step", C.c_uint64)]

    def as_dict(self) -> dict:
        return {"momentum": list(self.momentum), "kinetic_energy": self.kinetic_energy,
                "potential_energy": self.potential_energy, "mean_rho": self.mean_rho, "min_rho": self.min_rho,
                "max_rho": self.max_rho, "mean_abs_rho_dev": self.mean_abs_rho_dev,
                "nonfinite": int(self.nonfinite), "n": int(self.n), "step": int(self.step)}


class LearnedReport(C.Structure):
    _fields_ = [("learned_macro_steps", C.c_uint64), ("plain_macro_steps", C.c_uint64), ("judged", C.c_uint64),
                ("fallbacks", C.c_uint64), ("last_density_dev", C.c_double), ("last_momentum_dev", C.c_double),
                ("max_density_dev", C.c_double), ("sum_density_dev", C.c_double),
                ("discarded_macro_steps", C.c_uint64), ("last_mean_rho_dev", C.c_double),
                ("max_mean_rho_dev", C.c_double), ("last_max_rho_dev", C.c_double),
                ("max_max_rho_dev", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class View(C.Structure):
    """sph_view: camera, light, material and image size of sph_render."""
    _fields_ = [("model", C.c_float * 16), ("view", C.c_float * 16), ("proj", C.c_float * 16),
                ("eye_w", C.c_float * 4), ("light_w", C.c_float * 4), ("dark", C.c_float * 4),
                ("midtone", C.c_float * 4), ("highlight", C.c_float * 4), ("outline", C.c_float * 4),
                ("clear_color", C.c_float * 4), ("shininess", C.c_float), ("point_size", C.c_float),
                ("width", C.c_int32), ("height", C.c_int32)]


assert C.sizeof(View) == 320


# Every symbol of include/sph_gb300.h with its ctypes signature.
_P = C.c_void_p
_SIGS = {
    "sph_version": (C.c_char_p, []),
    "sph_params_default": (None, [C.POINTER(Params)]),
    "sph_params_validate": (C.c_int32, [C.POINTER(Params)]),
    "sph_cutoff_d2": (C.c_float, [C.c_float]),
    "sph_grid_dims": (C.c_int32, [C.POINTER(Params), C.POINTER(C.c_float), C.POINTER(C.c_int32)]),
    "sph_create": (C.c_int32, [C.POINTER(Params), C.c_uint32, _P, C.POINTER(_P)]),
    "sph_create_batch": (C.c_int32, [C.POINTER(Params), C.POINTER(C.c_uint32), C.c_uint32, _P, C.POINTER(_P)]),
    "sph_destroy": (C.c_int32, [_P]),
    "sph_last_error": (C.c_char_p, [_P]),
    "sph_set_params": (C.c_int32, [_P, C.POINTER(Params)]),
    "sph_get_params": (C.c_int32, [_P, C.POINTER(Params)]),
    "sph_upload_aos": (C.c_int32, [_P, _P, C.c_uint32]),
    "sph_download_aos": (C.c_int32, [_P, _P, C.c_uint32]),
    "sph_upload_aos_device": (C.c_int32, [_P, _P, C.c_uint32]),
    "sph_download_aos_device": (C.c_int32, [_P, _P, C.c_uint32]),
    "sph_step": (C.c_int32, [_P, C.c_int32]),
    "sph_synchronize": (C.c_int32, [_P]),
    "sph_reduce": (C.c_int32, [_P, C.POINTER(Diag)]),
    "sph_reduce_scenes": (C.c_int32, [_P, C.POINTER(Diag), C.c_uint32]),
    "sph_num_particles": (C.c_uint32, [_P]),
    "sph_num_scenes": (C.c_uint32, [_P]),
    "sph_step_count": (C.c_uint64, [_P]),
    "sph_enable_timing": (C.c_int32, [_P, C.c_int32]),
    "sph_pass_times": (C.c_int32, [_P, C.POINTER(C.c_float)]),
    "sph_neighbor_digest": (C.c_int32, [_P, _P, C.c_uint32, C.c_int32, _P, _P]),
    "sph_step_neighbor_digest": (C.c_int32, [_P, _P, C.c_uint32, _P, _P]),
    "sph_set_launch": (C.c_int32, [_P, C.c_int32, C.c_int32]),
    "sph_get_launch": (C.c_int32, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "sph_autotune": (C.c_int32, [_P, C.c_int32, C.POINTER(C.c_float)]),
    "sph_tile_stats": (C.c_int32, [_P, C.POINTER(C.c_uint32)]),
    "sph_record_stats": (C.c_int32, [_P, C.POINTER(C.c_uint64)]),
    "sph_set_record_mode": (C.c_int32, [_P, C.c_int32]),
    "sph_reduce_aos_noalloc": (C.c_int32, [_P, C.c_uint32, C.POINTER(Params), _P, _P]),
    "sph_mpnn_num_params": (C.c_uint32, []),
    "sph_mpnn_create": (C.c_int32, [C.c_uint32, _P, C.POINTER(_P)]),
    "sph_mpnn_destroy": (C.c_int32, [_P]),
    "sph_mpnn_last_error": (C.c_char_p, [_P]),
    "sph_mpnn_set_params": (C.c_int32, [_P, _P, C.c_uint32]),
    "sph_mpnn_get_params": (C.c_int32, [_P, _P, C.c_uint32]),
    "sph_mpnn_loss_grad": (C.c_int32, [_P, C.c_uint32, _P, _P, _P, _P, _P, _P, _P, C.POINTER(C.c_double), _P, _P]),
    "sph_mpnn_forward": (C.c_int32, [_P, C.c_uint32, _P, _P, _P, _P, _P, _P, C.c_int32, _P]),
    "sph_mpnn_set_precision": (C.c_int32, [_P, C.c_int32]),
    "sph_mpnn_set_train_precision": (C.c_int32, [_P, C.c_int32]),
    "sph_tc_gemm_bf16": (C.c_int32, [_P, _P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P]),
    "sph_mpnn_record": (C.c_int32, [_P, _P, C.c_uint32, C.POINTER(C.c_uint32)]),
    "sph_mpnn_clear_frames": (C.c_int32, [_P]),
    "sph_mpnn_train": (C.c_int32, [_P, C.c_uint32, C.c_float, C.c_uint64, _P]),
    "sph_learned_step": (C.c_int32, [_P, _P, C.c_int32, C.c_int32, C.c_float, C.c_float, C.POINTER(LearnedReport)]),
    "sph_refresh_density": (C.c_int32, [_P]),
    "sph_learned_set_judge": (C.c_int32, [_P, C.c_int32]),
    "sph_learned_set_max_density_tol": (C.c_int32, [_P, C.c_float]),
    "sph_neighbor_lists": (C.c_int32, [_P, _P, _P, _P]),
    "sph_view_default": (C.c_int32, [C.POINTER(View), C.c_int32, C.c_int32, C.c_float]),
    "sph_view_camera": (C.c_int32, [C.POINTER(View), C.c_float, C.c_float, C.POINTER(C.c_float),
                                    C.POINTER(C.c_float)]),
    "sph_render": (C.c_int32, [_P, C.POINTER(View), C.c_uint32, _P, C.c_int32]),
    "sph_image_write_ppm": (C.c_int32, [C.c_char_p, _P, C.c_int32, C.c_int32]),
    "sph_snapshot_save": (C.c_int32, [_P, C.c_char_p, C.c_uint64]),
    "sph_snapshot_info": (C.c_int32, [C.c_char_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32),
                                      C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
    "sph_snapshot_verify": (C.c_int32, [C.c_char_p]),
    "sph_snapshot_load": (C.c_int32, [C.c_char_p, _P, C.POINTER(_P)]),
    "sph_trajectory_create": (C.c_int32, [_P, C.c_char_p, C.c_uint64, C.POINTER(_P)]),
    "sph_trajectory_append": (C.c_int32, [_P, _P]),
    "sph_trajectory_frames": (C.c_uint64, [_P]),
    "sph_trajectory_close": (C.c_int32, [_P]),
    "sph_checksum64": (C.c_uint64, [_P, C.c_uint64]),
    "sph_scene_reference_grid": (C.c_int32, [_P, C.c_uint32, C.c_float]),
    "sph_scene_fill": (C.c_int32, [_P, C.c_uint32, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_float,
                                   C.c_float, C.c_uint64]),
    "sph_scene_ball": (C.c_int32, [_P, C.c_uint32, C.POINTER(C.c_float), C.c_float, C.c_float, C.c_uint64]),
    "sph_scene_slosh": (C.c_int32, [_P, C.c_uint32, C.c_float, C.c_float, C.c_float]),
    "sph_pair_counts": (C.c_int32, [_P, C.POINTER(C.c_uint64)]),
    "sph_set_obstacle": (C.c_int32, [_P, _P, C.POINTER(C.c_int32), C.POINTER(C.c_float), C.c_float]),
    "sph_sdf_from_mesh": (C.c_int32, [_P, C.c_uint32, _P, C.c_uint32, C.POINTER(C.c_int32), C.POINTER(C.c_float),
                                      C.c_float, _P]),
    "sph_obj_read": (C.c_int32, [C.c_char_p, _P, C.POINTER(C.c_uint32), _P, C.POINTER(C.c_uint32)]),
}


def _load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is not built: run `python npr-sph_gb300/build.py`")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


class SphError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"sph status {code}: {msg}")
        self.code = code


def _check(code: int, ctx=None, what: str = "") -> None:
    if code != OK:
        msg = lib.sph_last_error(ctx).decode() if ctx else what
        raise SphError(code, msg or what)


def _f3(v) -> C.Array:
    return (C.c_float * 3)(*[float(x) for x in v])


def default_params() -> Params:
    """The reference's literal uniforms and shader constants."""
    p = Params()
    lib.sph_params_default(C.byref(p))
    return p


def cutoff_d2(h: float) -> float:
    return float(lib.sph_cutoff_d2(C.c_float(h)))


def grid_dims(p: Params) -> tuple[float, tuple[int, int, int]]:
    e = C.c_float()
    d = (C.c_int32 * 3)()
    _check(lib.sph_grid_dims(C.byref(p), C.byref(e), d), what="sph_grid_dims")
    return float(e.value), (d[0], d[1], d[2])


def to_bf16_bits(a: np.ndarray) -> np.ndarray:
    """float32 -> bf16 bit patterns (uint16), round to nearest even (finite inputs)."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def bf16_bits_to_f32(b: np.ndarray) -> np.ndarray:
    return (np.asarray(b, dtype=np.uint32) << 16).view(np.float32)


def tc_gemm(a_bits: np.ndarray, b_bits: np.ndarray, splits: int = 1) -> np.ndarray:
    """D = A B^T on the tensor cores (sph_tc_gemm_bf16): A (m x k), B (n x k) bf16 bits;
    returns (splits, m, n) FP32 partials."""
    a = np.ascontiguousarray(a_bits, dtype=np.uint16)
    b = np.ascontiguousarray(b_bits, dtype=np.uint16)
    m, k = a.shape
    n = b.shape[0]
    d = np.zeros((splits, m, n), dtype=np.float32)
    _check(lib.sph_tc_gemm_bf16(a.ctypes.data, b.ctypes.data, m, n, k, splits, d.ctypes.data), what="sph_tc_gemm_bf16")
    return d


def empty_particles(n: int) -> np.ndarray:
    return np.zeros(n, dtype=PARTICLE_DTYPE)


# ---- views and images (sph_render) -----------------------------------------------------------

def view_default(width: int = 720, height: int = 720, model_scale: float = 1.0) -> View:
    v = View()
    _check(lib.sph_view_default(C.byref(v), width, height, model_scale), what="sph_view_default")
    return v


def view_camera(v: View, angle: float, scale: float, eye, center) -> View:
    _check(lib.sph_view_camera(C.byref(v), angle, scale, _f3(eye), _f3(center)), what="sph_view_camera")
    return v


def write_ppm(path, rgba: np.ndarray) -> None:
    rgba = np.ascontiguousarray(rgba, dtype=np.uint8)
    h, w, _ = rgba.shape
    _check(lib.sph_image_write_ppm(str(path).encode(), rgba.ctypes.data, w, h), what="sph_image_write_ppm")


# ---- snapshot and trajectory files (format in include/sph_gb300.h) --------------------------

_HEADER_DTYPE = np.dtype([("magic", "S8"), ("version", "<u4"), ("header_bytes", "<u4"), ("n", "<u8"),
                          ("scenes", "<u4"), ("flags", "<u4"), ("steps", "<u8"), ("seed", "<u8"),
                          ("checksum", "<u8"), ("reserved1", "<u8")])
_FRAME_HEAD = np.dtype([("step", "<u8"), ("n", "<u8"), ("checksum", "<u8"), ("reserved", "<u8")])


def checksum64(data) -> int:
    """FNV-1a 64 over 64-bit little-endian words (sph_checksum64)."""
    b = np.ascontiguousarray(np.frombuffer(memoryview(data).cast("B"), dtype=np.uint8))
    return int(lib.sph_checksum64(b.ctypes.data, b.nbytes))


def _read_head(raw: np.ndarray, magic: bytes):
    h = raw[:64].view(_HEADER_DTYPE)[0]
    if h["magic"] != magic or h["version"] != 1 or h["header_bytes"] != 64:
        raise ValueError("not a %s file" % magic.decode())
    scenes = int(h["scenes"])
    tb = (scenes * (96 + 4) + 63) // 64 * 64
    table = raw[64:64 + tb]
    params = [Params.from_buffer_copy(table[96 * i:96 * (i + 1)].tobytes()) for i in range(scenes)]
    counts = table[96 * scenes:96 * scenes + 4 * scenes].view("<u4").copy()
    return h, params, counts, 64 + tb


def snapshot_info(path) -> dict:
    n, sc, steps, seed = C.c_uint64(), C.c_uint32(), C.c_uint64(), C.c_uint64()
    _check(lib.sph_snapshot_info(str(path).encode(), C.byref(n), C.byref(sc), C.byref(steps), C.byref(seed)),
           what="sph_snapshot_info")
    return {"n": n.value, "scenes": sc.value, "steps": steps.value, "seed": seed.value}


def snapshot_verify(path) -> bool:
    return lib.sph_snapshot_verify(str(path).encode()) == 0


def read_snapshot(path) -> dict:
    """Header, uniforms, scene counts and records of a snapshot file (numpy, no GPU)."""
    raw = np.fromfile(path, dtype=np.uint8)
    h, params, counts, off = _read_head(raw, b"NPRSPHS1")
    n = int(h["n"])
    recs = raw[off:off + 64 * n].view(PARTICLE_DTYPE)
    if len(recs) != n:
        raise ValueError("truncated snapshot")
    order = None
    if int(h["flags"]) & 1:
        order = raw[off + 64 * n:off + 68 * n].view("<u4")
        if len(order) != n:
            raise ValueError("truncated snapshot")
    return {"n": n, "steps": int(h["steps"]), "seed": int(h["seed"]), "checksum": int(h["checksum"]),
            "params": params, "counts": counts, "particles": recs, "slot_order": order}


def read_trajectory(path) -> dict:
    """Header, uniforms, scene counts and frames [(step, records)] of a trajectory file."""
    raw = np.fromfile(path, dtype=np.uint8)
    h, params, counts, off = _read_head(raw, b"NPRSPHT1")
    n = int(h["n"])
    frames = []
    while off + 32 <= len(raw):
        fh = raw[off:off + 32].view(_FRAME_HEAD)[0]
        if int(fh["n"]) != n or off + 32 + 64 * n > len(raw):
            raise ValueError("truncated or inconsistent frame")
        recs = raw[off + 32:off + 32 + 64 * n].view(PARTICLE_DTYPE)
        if checksum64(recs) != int(fh["checksum"]):
            raise ValueError("frame checksum mismatch at step %d" % int(fh["step"]))
        frames.append((int(fh["step"]), recs))
        off += 32 + 64 * n
    return {"n": n, "seed": int(h["seed"]), "params": params, "counts": counts, "frames": frames}


class Trajectory:
    """Append-only trajectory file of a context (sph_trajectory_*)."""

    def __init__(self, sim: "Sim", path, seed: int = 0):
        self._t = C.c_void_p()
        _check(lib.sph_trajectory_create(sim.ctx, str(path).encode(), int(seed), C.byref(self._t)), sim.ctx)

    def append(self, sim: "Sim") -> None:
        _check(lib.sph_trajectory_append(self._t, sim.ctx), sim.ctx)

    @property
    def frames(self) -> int:
        return int(lib.sph_trajectory_frames(self._t))

    def close(self) -> None:
        if self._t:
            _check(lib.sph_trajectory_close(self._t), what="sph_trajectory_close")
            self._t = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def _ptr(a) -> int:
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("particle array must be C-contiguous")
        return a.ctypes.data
    return int(a.data_ptr())  # a torch tensor (device or pinned host)


class Sim:
    """One simulation context (single scene, or a batch of scenes)."""

    def __init__(self, params, n_max: int | None = None, counts=None, stream=None):
        self._ctx = C.c_void_p()
        s = C.c_void_p(int(stream) if stream is not None else 0)
        if counts is None:
            _check(lib.sph_create(C.byref(params), int(n_max), s, C.byref(self._ctx)), what="sph_create")
            self.n_scene = 1
        else:
            counts = np.ascontiguousarray(counts, dtype=np.uint32)
            plist = (Params * len(counts))(*params)
            _check(lib.sph_create_batch(plist, counts.ctypes.data_as(C.POINTER(C.c_uint32)), len(counts), s,
                                        C.byref(self._ctx)), what="sph_create_batch")
            self.n_scene = len(counts)
            self._counts = counts

    @classmethod
    def from_snapshot(cls, path, stream=None) -> "Sim":
        """A context restored from a snapshot file (sph_snapshot_load)."""
        obj = cls.__new__(cls)
        obj._ctx = C.c_void_p()
        s = C.c_void_p(int(stream) if stream is not None else 0)
        _check(lib.sph_snapshot_load(str(path).encode(), s, C.byref(obj._ctx)), what="sph_snapshot_load")
        obj.n_scene = int(lib.sph_num_scenes(obj._ctx))
        return obj

    def render(self, view: View, scene: int = 0, out: np.ndarray | None = None) -> np.ndarray:
        """Toon render of the particles (sph_render): (height, width, 4) uint8, rows bottom to top."""
        if out is None:
            out = np.zeros((view.height, view.width, 4), dtype=np.uint8)
        assert out.shape == (view.height, view.width, 4) and out.dtype == np.uint8 and out.flags.c_contiguous
        _check(lib.sph_render(self._ctx, C.byref(view), int(scene), out.ctypes.data, 0), self._ctx)
        return out

    def render_device(self, view: View, dev_ptr: int, scene: int = 0) -> None:
        """sph_render into a device buffer of width * height * 4 bytes."""
        _check(lib.sph_render(self._ctx, C.byref(view), int(scene), C.c_void_p(dev_ptr), 1), self._ctx)

    def set_obstacle(self, sdf: np.ndarray | None, origin=(0.0, 0.0, 0.0), spacing: float = 1.0) -> None:
        """Static obstacle from signed distance samples sdf[z, y, x] (sph_set_obstacle); None removes it."""
        if sdf is None:
            _check(lib.sph_set_obstacle(self._ctx, None, None, None, C.c_float(0.0)), self._ctx)
            return
        a = np.ascontiguousarray(sdf, dtype=np.float32)
        assert a.ndim == 3
        dims = (C.c_int32 * 3)(a.shape[2], a.shape[1], a.shape[0])
        _check(lib.sph_set_obstacle(self._ctx, a.ctypes.data, dims, _f3(origin), C.c_float(spacing)), self._ctx)

    def save(self, path, seed: int = 0) -> None:
        """Write a snapshot file (sph_snapshot_save)."""
        _check(lib.sph_snapshot_save(self._ctx, str(path).encode(), int(seed)), self._ctx)

    def close(self) -> None:
        if self._ctx:
            lib.sph_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def ctx(self):
        return self._ctx

    @property
    def n(self) -> int:
        return int(lib.sph_num_particles(self._ctx))

    @property
    def steps(self) -> int:
        return int(lib.sph_step_count(self._ctx))

    def set_params(self, p: Params) -> None:
        _check(lib.sph_set_params(self._ctx, C.byref(p)), self._ctx)

    def get_params(self) -> Params:
        p = Params()
        _check(lib.sph_get_params(self._ctx, C.byref(p)), self._ctx)
        return p

    def upload(self, particles: np.ndarray) -> None:
        _check(lib.sph_upload_aos(self._ctx, _ptr(particles), len(particles)), self._ctx)

    def download(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = empty_particles(self.n)
        _check(lib.sph_download_aos(self._ctx, _ptr(out), len(out)), self._ctx)
        return out

    def upload_device(self, dev_ptr: int, n: int) -> None:
        _check(lib.sph_upload_aos_device(self._ctx, C.c_void_p(dev_ptr), n), self._ctx)

    def download_device(self, dev_ptr: int, n: int) -> None:
        _check(lib.sph_download_aos_device(self._ctx, C.c_void_p(dev_ptr), n), self._ctx)

    def step(self, n: int = 1) -> None:
        _check(lib.sph_step(self._ctx, int(n)), self._ctx)

    def synchronize(self) -> None:
        _check(lib.sph_synchronize(self._ctx), self._ctx)

    def reduce(self) -> Diag:
        d = Diag()
        _check(lib.sph_reduce(self._ctx, C.byref(d)), self._ctx)
        return d

    def reduce_scenes(self) -> list[Diag]:
        arr = (Diag * self.n_scene)()
        _check(lib.sph_reduce_scenes(self._ctx, arr, self.n_scene), self._ctx)
        return list(arr)

    def enable_timing(self, on: bool = True) -> None:
        _check(lib.sph_enable_timing(self._ctx, 1 if on else 0), self._ctx)

    def pass_times(self) -> list[float]:
        a = (C.c_float * 3)()
        _check(lib.sph_pass_times(self._ctx, a), self._ctx)
        return [a[0], a[1], a[2]]

    def neighbor_digest(self, query_ids, brute_force: bool = False):
        q = np.ascontiguousarray(query_ids, dtype=np.uint32)
        cnt = np.zeros(len(q), dtype=np.uint32)
        dig = np.zeros(len(q), dtype=np.uint64)
        _check(lib.sph_neighbor_digest(self._ctx, q.ctypes.data, len(q), 1 if brute_force else 0, cnt.ctypes.data,
                                       dig.ctypes.data), self._ctx)
        return cnt, dig

    def step_neighbor_digest(self, query_ids):
        """One plain step that reports the neighbour sets its force pass used for the query
        particles (count with self, digest), as neighbor_digest reports them before the step."""
        q = np.ascontiguousarray(query_ids, dtype=np.uint32)
        cnt = np.zeros(len(q), dtype=np.uint32)
        dig = np.zeros(len(q), dtype=np.uint64)
        _check(lib.sph_step_neighbor_digest(self._ctx, q.ctypes.data, len(q), cnt.ctypes.data, dig.ctypes.data),
               self._ctx)
        return cnt, dig

    def set_launch(self, threads_per_block: int, stencil: int) -> None:
        _check(lib.sph_set_launch(self._ctx, threads_per_block, stencil), self._ctx)

    def get_launch(self) -> tuple[int, int]:
        a, b = C.c_int32(), C.c_int32()
        _check(lib.sph_get_launch(self._ctx, C.byref(a), C.byref(b)), self._ctx)
        return a.value, b.value

    def pair_counts(self) -> tuple[int, int]:
        """(candidate tests of the density pass, pairs with r < h incl. self) of the next step at
        the current positions (sph_pair_counts)."""
        out = (C.c_uint64 * 2)()
        _check(lib.sph_pair_counts(self._ctx, out), self._ctx)
        return int(out[0]), int(out[1])

    def record_stats(self) -> tuple[int, int, int]:
        """(steps with, steps without) the force pass's 32-byte neighbour records since creation,
        and the same-cell pairs (sum of count^2 over the cells) the last sort seen by the host
        found (sph_record_stats)."""
        a = (C.c_uint64 * 3)()
        _check(lib.sph_record_stats(self._ctx, a), self._ctx)
        return int(a[0]), int(a[1]), int(a[2])

    def set_record_mode(self, mode: int) -> None:
        """0: neighbour records chosen per step (default), 1: always, 2: never (sph_set_record_mode)."""
        _check(lib.sph_set_record_mode(self._ctx, int(mode)), self._ctx)

    def tile_stats(self) -> tuple[int, int]:
        """(density, force) chunks that fell back to the global-memory path since creation."""
        a = (C.c_uint32 * 2)()
        _check(lib.sph_tile_stats(self._ctx, a), self._ctx)
        return a[0], a[1]

    def autotune(self, trial_steps: int = 5) -> float:
        ms = C.c_float()
        _check(lib.sph_autotune(self._ctx, trial_steps, C.byref(ms)), self._ctx)
        return float(ms.value)


    def neighbor_lists(self):
        """(nb (n, 32) ids, counts (n,), rho (n,)) by particle id (sph_neighbor_lists)."""
        n = self.n
        nb = np.zeros((n, 32), np.int32)
        cnt = np.zeros(n, np.int32)
        rho = np.zeros(n, np.float32)
        _check(lib.sph_neighbor_lists(self._ctx, nb.ctypes.data, cnt.ctypes.data, rho.ctypes.data), self._ctx)
        return nb, cnt, rho

    def refresh_density(self) -> None:
        """rho and pres at the current positions (sph_refresh_density)."""
        _check(lib.sph_refresh_density(self._ctx), self._ctx)

    def set_judge(self, metric: int) -> None:
        """Density deviation of the learned step's judge: JUDGE_MEAN_DENSITY or JUDGE_PARTICLE_DENSITY."""
        _check(lib.sph_learned_set_judge(self._ctx, metric), self._ctx)

    def set_max_density_tol(self, tol: float) -> None:
        """Bound of the judge on the deviation of the maximum density (sph_learned_set_max_density_tol)."""
        _check(lib.sph_learned_set_max_density_tol(self._ctx, C.c_float(tol)), self._ctx)

    def learned_step(self, net: "Net", n_macro: int, judge_every: int = 8, density_tol: float = 0.01,
                     momentum_tol: float = 0.01) -> LearnedReport:
        rep = LearnedReport()
        _check(lib.sph_learned_step(self._ctx, net.handle, n_macro, judge_every, density_tol, momentum_tol,
                                    C.byref(rep)), self._ctx)
        return rep


class Net:
    """The learned macro-step network (sph_mpnn_*): parameters, training frames, training."""

    def __init__(self, n_frame: int, stream=None):
        self._h = C.c_void_p()
        s = C.c_void_p(int(stream) if stream is not None else 0)
        _check(lib.sph_mpnn_create(n_frame, s, C.byref(self._h)), what="sph_mpnn_create")
        self.n_params = int(lib.sph_mpnn_num_params())

    @property
    def handle(self):
        return self._h

    def _check(self, code):
        if code != OK:
            raise SphError(code, lib.sph_mpnn_last_error(self._h).decode())

    def close(self):
        if self._h:
            lib.sph_mpnn_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_params(self, flat: np.ndarray) -> None:
        a = np.ascontiguousarray(flat, dtype=np.float32)
        self._check(lib.sph_mpnn_set_params(self._h, a.ctypes.data, len(a)))

    def get_params(self) -> np.ndarray:
        a = np.zeros(self.n_params, dtype=np.float32)
        self._check(lib.sph_mpnn_get_params(self._h, a.ctypes.data, len(a)))
        return a

    def loss_grad(self, pos4, vel4, rhop2, nb, cnt, target8, fc):
        """Loss, outputs (n x 8) and gradient of one host frame (sph_mpnn_loss_grad)."""
        n = len(pos4)
        arrs = [np.ascontiguousarray(x, dtype=t) for x, t in
                ((pos4, np.float32), (vel4, np.float32), (rhop2, np.float32), (nb, np.int32), (cnt, np.int32),
                 (target8, np.float32), (fc, np.float32))]
        assert arrs[5].shape == (n, 8) and arrs[6].shape == (6,)
        out = np.zeros((n, 8), dtype=np.float32)
        grad = np.zeros(self.n_params, dtype=np.float32)
        loss = C.c_double()
        self._check(lib.sph_mpnn_loss_grad(self._h, n, *[a.ctypes.data for a in arrs], C.byref(loss), out.ctypes.data,
                                           grad.ctypes.data))
        return loss.value, out, grad

    def forward(self, pos4, vel4, rhop2, nb, cnt, fc, precision: int = 1) -> np.ndarray:
        """Network outputs (n x 8: O_v, O_x, 0, 0) of a host frame (sph_mpnn_forward)."""
        n = len(pos4)
        arrs = [np.ascontiguousarray(x, dtype=t) for x, t in
                ((pos4, np.float32), (vel4, np.float32), (rhop2, np.float32), (nb, np.int32), (cnt, np.int32),
                 (fc, np.float32))]
        assert arrs[5].shape == (6,)
        out = np.zeros((n, 8), dtype=np.float32)
        self._check(lib.sph_mpnn_forward(self._h, n, *[a.ctypes.data for a in arrs], precision, out.ctypes.data))
        return out

    def set_precision(self, precision: int) -> None:
        self._check(lib.sph_mpnn_set_precision(self._h, precision))

    def set_train_precision(self, precision: int) -> None:
        """1: node layers of the training passes on the BF16 tensor cores (default); 0: FP32."""
        self._check(lib.sph_mpnn_set_train_precision(self._h, precision))

    def record(self, sim: Sim, n_frames: int) -> int:
        tot = C.c_uint32()
        self._check(lib.sph_mpnn_record(self._h, sim.ctx, n_frames, C.byref(tot)))
        return tot.value

    def clear_frames(self) -> None:
        self._check(lib.sph_mpnn_clear_frames(self._h))

    def train(self, steps: int, lr: float = 1e-3, seed: int = 0) -> np.ndarray:
        losses = np.zeros(steps, dtype=np.float32)
        self._check(lib.sph_mpnn_train(self._h, steps, C.c_float(lr), C.c_uint64(seed), losses.ctypes.data))
        return losses


# ---- scenes -------------------------------------------------------------------------------

def scene_reference_grid() -> np.ndarray:
    """make_grid()+init_particles() of Main.cpp:488-539 (10x100x10 lattice at 0.005)."""
    a = empty_particles(10000)
    _check(lib.sph_scene_reference_grid(_ptr(a), 10000, C.c_float(0.005)), what="sph_scene_reference_grid")
    return a


def scene_fill(n: int, lo, hi, spacing: float, jitter: float, seed: int) -> np.ndarray:
    a = empty_particles(n)
    _check(lib.sph_scene_fill(_ptr(a), n, _f3(lo), _f3(hi), C.c_float(spacing), C.c_float(jitter),
                              C.c_uint64(seed)), what="sph_scene_fill")
    return a


def scene_ball(n: int, center, spacing: float, jitter: float, seed: int) -> np.ndarray:
    a = empty_particles(n)
    _check(lib.sph_scene_ball(_ptr(a), n, _f3(center), C.c_float(spacing), C.c_float(jitter), C.c_uint64(seed)),
           what="sph_scene_ball")
    return a


def scene_slosh(a: np.ndarray, amplitude: float, x0: float, length: float) -> np.ndarray:
    _check(lib.sph_scene_slosh(_ptr(a), len(a), C.c_float(amplitude), C.c_float(x0), C.c_float(length)),
           what="sph_scene_slosh")
    return a


def sdf_from_mesh(verts: np.ndarray, tris: np.ndarray, dims, origin, spacing: float) -> np.ndarray:
    """Signed distance samples [z, y, x] of a closed triangle mesh on a grid (sph_sdf_from_mesh, GPU)."""
    v = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(tris, dtype=np.uint32).reshape(-1, 3)
    nx, ny, nz = (int(d) for d in dims)
    out = np.zeros((nz, ny, nx), dtype=np.float32)
    _check(lib.sph_sdf_from_mesh(v.ctypes.data, len(v), t.ctypes.data, len(t), (C.c_int32 * 3)(nx, ny, nz),
                                 _f3(origin), C.c_float(spacing), out.ctypes.data), what="sph_sdf_from_mesh")
    return out


def obj_read(path) -> tuple[np.ndarray, np.ndarray]:
    """Vertices (n, 3) float32 and triangles (m, 3) uint32 of a Wavefront OBJ file (sph_obj_read)."""
    nv, nt = C.c_uint32(0), C.c_uint32(0)
    _check(lib.sph_obj_read(str(path).encode(), None, C.byref(nv), None, C.byref(nt)), what="sph_obj_read")
    v = np.zeros((nv.value, 3), dtype=np.float32)
    t = np.zeros((nt.value, 3), dtype=np.uint32)
    _check(lib.sph_obj_read(str(path).encode(), v.ctypes.data, C.byref(nv), t.ctypes.data, C.byref(nt)),
           what="sph_obj_read")
    return v, t


def icosphere(radius: float = 1.0, center=(0.0, 0.0, 0.0), subdivisions: int = 2) -> tuple[np.ndarray, np.ndarray]:
    """A closed triangle mesh of a sphere (an icosahedron with each face split in 4, `subdivisions`
    times, vertices pushed onto the sphere), counter-clockwise seen from outside."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    for _ in range(subdivisions):
        mid: dict = {}

        def midpoint(a: int, b: int) -> int:
            key = (min(a, b), max(a, b))
            if key not in mid:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                mid[key] = len(verts) - 1
            return mid[key]

        nf = []
        for a, b, c in f:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = nf
    return (radius * np.array(verts) + np.asarray(center, dtype=np.float64)).astype(np.float32), \
        np.array(f, dtype=np.uint32)


def write_obj(path, verts: np.ndarray, tris: np.ndarray) -> None:
    with open(path, "w") as fh:
        for x, y, z in verts:
            fh.write(f"v {x:.9g} {y:.9g} {z:.9g}\n")
        for a, b, c in tris:
            fh.write(f"f {a + 1} {b + 1} {c + 1}\n")


def workload_params(gravity_y: float = -9.81, dt: float = 1e-4, lower=None, upper=None, k=None, mu=None,
                    flags: int = 0) -> Params:
    """The benchmark scenes' uniforms: the reference's m, h, rho0, k, mu and damping, with
    gravity (0, -9.81, 0) and a fixed dt of 1e-4 (the shader's 1/NUM_PARTICLES at 10k)."""
    p = default_params()
    p.gravity[1] = gravity_y
    p.dt = dt
    if lower is not None:
        for a in range(3):
            p.lower[a] = lower[a]
    if upper is not None:
        for a in range(3):
            p.upper[a] = upper[a]
    if k is not None:
        p.gas_const = k
    if mu is not None:
        p.visc = mu
    p.flags = flags
    return p


@dataclass
class Scene:
    name: str
    params: Params
    particles: np.ndarray
    steps: int


def reference_scene_10k(seed: int = 1) -> Scene:
    """10,000 particles on a 0.5h lattice (jitter +-0.01h) filling the lower-corner quarter
    (half of x, half of z, from the floor up) of the reference box; G = (0,-9.81,0); 200 steps."""
    p = workload_params()
    h = p.h
    lo = [p.lower[a] for a in range(3)]
    hi = [p.lower[0] + 0.5 * (p.upper[0] - p.lower[0]), p.upper[1], p.lower[2] + 0.5 * (p.upper[2] - p.lower[2])]
    parts = scene_fill(10000, lo, hi, 0.5 * h, 0.01 * h, seed)
    return Scene("reference_10k", p, parts, 200)


def dam_break(nx: int = 64, ny: int = 128, nz: int = 128, seed: int = 2, flags: int = 0) -> Scene:
    """Dam break: an nx*ny*nz block (spacing 0.5h, jitter +-0.01h) against the x = 0 wall of a
    4:1:1 box whose y and z extents equal the block's (64x128x128 = 1,048,576 particles in
    5.12 x 1.28 x 1.28); 1,000 steps."""
    p0 = default_params()
    s = 0.5 * p0.h
    bx, by, bz = nx * s, ny * s, nz * s
    L = max(by, bz)
    p = workload_params(lower=(0.0, 0.0, 0.0), upper=(4 * L, by, bz), flags=flags)
    parts = scene_fill(nx * ny * nz, (0.0, 0.0, 0.0), (bx, by, bz), s, 0.01 * p.h, seed)
    return Scene(f"dam_break_{nx}x{ny}x{nz}", p, parts, 1000)


def slosh_block(n_side: int = 256, seed: int = 5) -> Scene:
    """n_side^3 block (spacing 0.5h) in a 2:1:1 box, v_x = 0.5 sin(pi x / L), L = box length."""
    p0 = default_params()
    s = 0.5 * p0.h
    b = n_side * s
    p = workload_params(lower=(0.0, 0.0, 0.0), upper=(2 * b, b, b))
    parts = scene_fill(n_side ** 3, (0.0, 0.0, 0.0), (b, b, b), s, 0.01 * p.h, seed)
    scene_slosh(parts, 0.5, 0.0, 2 * b)
    return Scene(f"slosh_{n_side}^3", p, parts, 2000)


def batched_scenes(n_scene: int = 256, seed: int = 3, n_lo: int = 2000, n_hi: int = 65536):
    """n_scene independent boxes: counts log-uniform in [n_lo, n_hi], k ~ U[500, 3000],
    mu ~ U[0.1, 2.0]; a coin flip picks a corner lattice or a sphere drop. Each box is a cube
    of edge 2 * cbrt(count) * spacing (fluid fills an eighth of it). Returns
    (params list, counts, concatenated particles)."""
    rng = np.random.default_rng(seed)
    p0 = default_params()
    s = 0.5 * p0.h
    plist, counts, parts = [], [], []
    for i in range(n_scene):
        cnt = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        k = float(rng.uniform(500.0, 3000.0))
        mu = float(rng.uniform(0.1, 2.0))
        ball = bool(rng.integers(0, 2))
        edge = 2.0 * math.ceil(cnt ** (1.0 / 3.0) + 1) * s
        p = workload_params(lower=(0.0, 0.0, 0.0), upper=(edge, edge, edge), k=k, mu=mu)
        if ball:
            a = scene_ball(cnt, (0.5 * edge, 0.6 * edge, 0.5 * edge), s, 0.01 * p.h, seed * 1000003 + i)
        else:
            a = scene_fill(cnt, (0.0, 0.0, 0.0), (0.5 * edge, edge, 0.5 * edge), s, 0.01 * p.h,
                           seed * 1000003 + i)
        plist.append(p)
        counts.append(cnt)
        parts.append(a)
    return plist, np.array(counts, dtype=np.uint32), np.concatenate(parts)
