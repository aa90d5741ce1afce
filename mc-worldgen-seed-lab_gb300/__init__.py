"""Python binding of libmcgen_gb300.so -- the GB300 biome engine behind libmcgen's C ABI.

Mirrors the reference's ctypes layer (blender/mcgen_addon/core/lib.py: ``load``, ``McError``,
``Generator.open(...).world(dimension, preset, seeds)``, ``World.biome_at`` / ``World.biome_grid``) so
callers and tests read like the reference's, plus the additions of include/mcgen_gb300.h (seeds x points,
quart grids with a tie rule, device-pointer forms).

The library is the product: loading fails loudly when libmcgen_gb300.so has not been built, and every
biome call raises McError when no CUDA device is usable.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmcgen_gb300.so")
DATA_ROOT = HERE  # data/climate-<V>.txt and data/params/<V>/ live under this directory

MCGEN_OK, MCGEN_E_ARG, MCGEN_E_IO, MCGEN_E_DATA, MCGEN_E_VERSION = 0, 1, 2, 3, 4
MCGEN_E_NOMEM, MCGEN_E_CANCEL, MCGEN_E_UNSUPPORTED, MCGEN_E_INTERNAL = 5, 6, 7, 8
MCGEN_COMPUTE_CPU, MCGEN_COMPUTE_GPU, MCGEN_COMPUTE_AUTO = 0, 1, 2
TIE_ENGINE, TIE_GRID_CHAIN, TIE_CHUNK_CELL, TIE_CHUNK_ORDER = 0, 1, 2, 3
PIPES = {"fp32_fma": 0, "fp64_fma": 1, "fp64_add": 2, "int32_mad": 3, "cvt_f64_floor_s32": 4,
         "cvt_s32_f64": 5, "cvt_f64_f32": 6, "int64_mad": 7, "cvt_s64_f64": 8, "cvt_f32_f64": 9}
ERR_BUF = 1024
_P = C.c_void_p


class McError(RuntimeError):
    def __init__(self, code: int, message: str, where: str = ""):
        super().__init__(f"{where}: {message} (code {code})" if where else f"{message} (code {code})")
        self.code = code
        self.where = where


class McSeeds(C.Structure):
    _fields_ = [("climate", C.c_int64), ("terrain", C.c_int64), ("structures", C.c_int64), ("features", C.c_int64)]


_PROTOS = {
    "mcgen_version": (C.c_char_p, []),
    "mcgen_abi_version": (C.c_int, []),
    "mcgen_open": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(_P), C.c_char_p, C.c_size_t]),
    "mcgen_close": (None, [_P]),
    "mcgen_dimension_count": (C.c_int, [_P]),
    "mcgen_dimension_name": (C.c_char_p, [_P, C.c_int]),
    "mcgen_preset_count": (C.c_int, [_P, C.c_char_p]),
    "mcgen_preset_name": (C.c_char_p, [_P, C.c_char_p, C.c_int]),
    "mcgen_block_state_count": (C.c_int, [_P]),
    "mcgen_biome_count": (C.c_int, [_P]),
    "mcgen_biome_name": (C.c_char_p, [_P, C.c_int]),
    "mcgen_tweak_count": (C.c_int, [_P]),
    "mcgen_world_new": (C.c_int, [_P, C.c_char_p, C.c_char_p, C.POINTER(McSeeds), _P, C.c_int, C.POINTER(_P),
                                  C.c_char_p, C.c_size_t]),
    "mcgen_world_free": (None, [_P]),
    "mcgen_world_min_y": (C.c_int, [_P]),
    "mcgen_world_height": (C.c_int, [_P]),
    "mcgen_world_sea_level": (C.c_int, [_P]),
    "mcgen_biome_at": (C.c_int, [_P, C.c_int, C.c_int, C.c_int]),
    "mcgen_biome_grid": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P]),
    "mcgen_gpu_biome_grid": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P]),
    "mcgen_biome_grid_cpu": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P]),
    "mcgen_gpu_biome_points": (C.c_int, [_P, C.c_int, _P, _P, C.POINTER(C.c_int)]),
    "mcgen_generate_region": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint32, C.c_int, _P, _P,
                                        C.POINTER(_P), C.c_char_p, C.c_size_t]),
    "mcgen_gpu_set_features": (C.c_int, [C.c_int]),
    "mcgen_gpu_get_features": (C.c_int, []),
    "mcgen_gpu_set_library_path": (C.c_int, [C.c_char_p]),
    "mcgen_gpu_device_count": (C.c_int, []),
    "mcgen_gpu_device_info": (C.c_int, [C.c_int, C.c_char_p, C.c_size_t, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                        C.POINTER(C.c_size_t)]),
    "mcgen_gpu_set_compute": (C.c_int, [C.c_int, C.c_int]),
    "mcgen_gpu_get_compute": (C.c_int, []),
    "mcgen_gpu_status": (C.c_int, [C.c_char_p, C.c_size_t]),
    "mcgen_gpu_selftest": (C.c_int, [_P, C.c_int, C.c_char_p, C.c_size_t]),
    "mcgen_gb300_world_info": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int64),
                                         C.POINTER(C.c_int)]),
    "mcgen_gb300_quart_grid": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P]),
    "mcgen_gb300_quart_grid_dev": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P]),
    "mcgen_gb300_seed_points": (C.c_int, [_P, _P, C.c_int, _P, C.c_int, _P, _P]),
    "mcgen_gb300_seed_points_dev": (C.c_int, [_P, _P, C.c_int, _P, C.c_int, _P, _P, _P]),
    "mcgen_gb300_biome_grid_dev": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P]),
    "mcgen_gb300_seed_points_noalloc": (C.c_int, [_P, _P, C.c_int, _P, C.c_int, _P, _P, _P]),
    "mcgen_gb300_launch_count": (C.c_longlong, []),
    "mcgen_gb300_last_error": (C.c_char_p, []),
    "mcgen_gb300_profile": (C.c_int, [C.c_int]),
    "mcgen_gb300_profile_read": (C.c_int, [C.c_int, C.POINTER(C.c_char_p), C.POINTER(C.c_double),
                                           C.POINTER(C.c_longlong)]),
    "mcgen_gb300_pipe_rate": (C.c_int, [C.c_int, C.POINTER(C.c_double)]),
    "mcgen_gb300_check_octave": (C.c_int, [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong)]),
    "mcgen_gb300_check_zoom": (C.c_int, [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong),
                                         C.POINTER(C.c_longlong)]),
    "mcgen_gb300_check_noise": (C.c_int, [_P, C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong),
                                          C.POINTER(C.c_longlong), C.POINTER(C.c_double)]),
    "mcgen_gb300_check_noise_quant": (C.c_int, [_P, C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong),
                                                C.POINTER(C.c_longlong), C.POINTER(C.c_double),
                                                C.POINTER(C.c_longlong)]),
    "mcgen_gb300_check_climate": (C.c_int, [_P, C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong),
                                            C.POINTER(C.c_longlong)]),
    "mcgen_gb300_check_tree": (C.c_int, [_P, C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong),
                                         C.POINTER(C.c_longlong)]),
    "mcgen_gb300_search": (C.c_int, [_P, C.c_int, _P, C.c_uint64, C.c_uint64, _P, C.c_int, C.c_int, _P, C.c_uint32,
                                     C.POINTER(C.c_uint32), _P, C.POINTER(C.c_double)]),
    "mcgen_gb300_obs_end_radius": (C.c_int, [_P, _P]),
    "mcgen_gb300_check_split": (C.c_int, [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_longlong),
                                          C.POINTER(C.c_longlong)]),
}

_PROTOS.update({
    "mcgen_gb300_quart_grid_seed_dev": (C.c_int, [_P, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                                  _P, _P]),
    "mcgen_gb300_plan_new": (C.c_int, [_P, C.c_int, C.c_int, C.POINTER(_P)]),
    "mcgen_gb300_plan_free": (None, [_P]),
    "mcgen_gb300_plan_output_bytes": (C.c_longlong, [_P]),
    "mcgen_gb300_plan_output_offset": (C.c_longlong, [_P, C.c_int]),
    "mcgen_gb300_plan_shape": (C.c_int, [_P]),
    "mcgen_gb300_plan_set_shape": (C.c_int, [_P, C.c_int]),
    "mcgen_gb300_plan_h2d_bytes": (C.c_longlong, [_P]),
    "mcgen_gb300_plan_autotune": (C.c_int, [_P, _P, C.c_int, C.POINTER(C.c_double)]),
    "mcgen_gb300_plan_run_dev": (C.c_int, [_P, _P, _P]),
    "mcgen_gb300_plan_run_dev_direct": (C.c_int, [_P, _P, _P]),
    "mcgen_gb300_plan_run": (C.c_int, [_P, _P]),
    "mcgen_gb300_server_new": (C.c_int, [C.c_longlong, C.c_int, C.c_int, C.POINTER(_P)]),
    "mcgen_gb300_server_free": (None, [_P]),
    "mcgen_gb300_server_submit": (C.c_int, [_P, _P, _P, C.POINTER(C.c_longlong)]),
    "mcgen_gb300_server_wait": (C.c_int, [_P, C.c_longlong, C.c_int, C.POINTER(C.c_double)]),
    "mcgen_gb300_server_stats": (C.c_int, [_P, _P]),
    "mcgen_gb300_server_fail_next": (C.c_int, [_P, C.c_int]),
    "mcgen_gb300_check_end": (C.c_int, [C.c_longlong, C.c_ulonglong, _P, _P, _P]),
    "mcgen_gb300_server_replay": (C.c_int, [_P, _P, _P, C.c_int, _P, _P, _P, _P]),
    "mcgen_gb300_density_values": (C.c_int, [_P, C.c_int64, C.c_int, _P, _P]),
    "mcgen_gb300_seed_points_noalloc": (C.c_int, [_P, _P, C.c_int, _P, C.c_int, _P, _P, _P]),
})


class McGb300ServerStats(C.Structure):
    _fields_ = [(n, C.c_longlong) for n in ("requests_submitted", "requests_admitted", "batches", "samples_done",
                                            "cache_hits", "cache_misses", "cache_evictions", "cache_entries",
                                            "pending")] + [("cache_slots", C.c_longlong * 3)]


class McGb300Request(C.Structure):
    _fields_ = [("world", _P), ("seed", C.c_int64), ("qx0", C.c_int32), ("qz0", C.c_int32), ("nx", C.c_int32),
                ("nz", C.c_int32), ("qy", C.c_int32)]


# McGb300Request as a numpy record, for building request lists without a per-request ctypes object
REQUEST_DTYPE = np.dtype([("world", np.uint64), ("seed", np.int64), ("qx0", np.int32), ("qz0", np.int32),
                          ("nx", np.int32), ("nz", np.int32), ("qy", np.int32)], align=True)
assert REQUEST_DTYPE.itemsize == C.sizeof(McGb300Request)


_lib = None


def load(path: str | None = None):
    """Load libmcgen_gb300.so (built in-tree by build.py).  Raises if it is missing: there is no fallback."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise McError(MCGEN_E_UNSUPPORTED, f"{p} not built (run the package's build.py)", "load")
    L = C.CDLL(p)
    for name, (res, args) in _PROTOS.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _check(rc: int, where: str, err=None):
    if rc != MCGEN_OK:
        msg = err.value.decode(errors="replace") if err is not None and err.value else ""
        if not msg:
            msg = (load().mcgen_gb300_last_error() or b"").decode(errors="replace") or "failed"
        raise McError(rc, msg, where)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_P)


def version_string() -> str:
    return load().mcgen_version().decode()


def device_count() -> int:
    return load().mcgen_gpu_device_count()


def gpu_status() -> tuple[bool, str]:
    buf = C.create_string_buffer(2048)
    ok = load().mcgen_gpu_status(buf, 2048)
    return bool(ok), buf.value.decode(errors="replace")


def launch_count() -> int:
    return load().mcgen_gb300_launch_count()


def profile(enable: bool) -> None:
    """Start (clearing) or stop per-kernel CUDA-event timing of the library's launches."""
    _check(load().mcgen_gb300_profile(1 if enable else 0), "mcgen_gb300_profile")


def profile_read() -> dict:
    """{kernel name: (total ms, launches)} for kernels launched while profiling was on."""
    L = load()
    out = {}
    k = 0
    while True:
        name, ms, n = C.c_char_p(), C.c_double(), C.c_longlong()
        if L.mcgen_gb300_profile_read(k, C.byref(name), C.byref(ms), C.byref(n)) != MCGEN_OK:
            break
        if n.value:
            out[name.value.decode()] = (ms.value, n.value)
        k += 1
    return out


def check_split(n: int, seed: int = 1) -> tuple[int, int]:
    """Mismatches (float branch, double branch) of the fast coordinate split against the plain one."""
    bf, bd = C.c_longlong(), C.c_longlong()
    _check(load().mcgen_gb300_check_split(n, seed, C.byref(bf), C.byref(bd)), "mcgen_gb300_check_split")
    return bf.value, bd.value


def check_octave(n: int, seed: int = 1) -> int:
    """Mismatches of the double branch's fixed-point octave against the plain double octave."""
    b = C.c_longlong()
    _check(load().mcgen_gb300_check_octave(n, seed, C.byref(b)), "mcgen_gb300_check_octave")
    return b.value


def check_zoom(n: int, seed: int = 1) -> tuple[int, int]:
    """(mismatches, cases decided in double precision) of the screened zoom choice against the plain one."""
    b, c = C.c_longlong(), C.c_longlong()
    _check(load().mcgen_gb300_check_zoom(n, seed, C.byref(b), C.byref(c)), "mcgen_gb300_check_zoom")
    return b.value, c.value


def check_end(n: int, seed: int = 1) -> tuple[int, int, float]:
    """(wrong decisions, cases left to the exact value, worst float error / bound) of the End's screened
    island test against the reference's double simplex."""
    b, c, r = C.c_longlong(), C.c_longlong(), C.c_double()
    _check(load().mcgen_gb300_check_end(n, seed, C.byref(b), C.byref(c), C.byref(r)), "mcgen_gb300_check_end")
    return b.value, c.value, r.value


def check_noise(world: "World", n: int, seed: int = 1) -> tuple[int, int, float]:
    """(mismatches, values left to the exact path, worst error / bound) of the double branch's screened
    climate noises against the exact double evaluation, on the world's own seed lattices."""
    b, c, r = C.c_longlong(), C.c_longlong(), C.c_double()
    _check(load().mcgen_gb300_check_noise(world.handle, n, seed, C.byref(b), C.byref(c), C.byref(r)),
           "mcgen_gb300_check_noise")
    return b.value, c.value, r.value


def check_noise_quant(world: "World", n: int, seed: int = 1) -> tuple[int, int, float, int]:
    """(target mismatches, values left to the 59-bit screen, worst error / bound, settled values near a target
    boundary) of the 32-bit screen of the double branch's quantised-only noises (temperature, vegetation)
    against the exact double evaluation, on the world's own seed lattices."""
    b, c, r, m = C.c_longlong(), C.c_longlong(), C.c_double(), C.c_longlong()
    _check(load().mcgen_gb300_check_noise_quant(world.handle, n, seed, C.byref(b), C.byref(c), C.byref(r),
                                                C.byref(m)), "mcgen_gb300_check_noise_quant")
    return b.value, c.value, r.value, m.value


def check_climate(world: "World", n: int, seed: int = 1) -> tuple[int, int]:
    """(cells whose targets differ, cells with a value the screen left to the exact path) of the double
    branch's Overworld climate as the kernels compute it against the plain double evaluation, on n random
    quart cells."""
    b, c = C.c_longlong(), C.c_longlong()
    _check(load().mcgen_gb300_check_climate(world.handle, n, seed, C.byref(b), C.byref(c)),
           "mcgen_gb300_check_climate")
    return b.value, c.value


def check_tree(world: "World", n: int, seed: int = 1) -> tuple[int, int]:
    """(differing leaves, differing fitness values or tie flags) of the 32-bit R-tree searches against the
    64-bit stack searches on n random targets of the world's tree."""
    b, c = C.c_longlong(), C.c_longlong()
    _check(load().mcgen_gb300_check_tree(world.handle, n, seed, C.byref(b), C.byref(c)), "mcgen_gb300_check_tree")
    return b.value, c.value


def pipe_rate(pipe: str) -> float:
    """Measured throughput of one GPU pipe in giga-operations per second (see PIPES)."""
    g = C.c_double()
    _check(load().mcgen_gb300_pipe_rate(PIPES[pipe], C.byref(g)), "mcgen_gb300_pipe_rate")
    return g.value


class Generator:
    """McGen: one version's data (mcgen_open)."""

    def __init__(self, handle, data_root: str, version: str):
        self._h = handle
        self.data_root = data_root
        self.version = version

    @classmethod
    def open(cls, data_root: str = DATA_ROOT, version: str = "26.3") -> "Generator":
        L = load()
        h = _P()
        err = C.create_string_buffer(ERR_BUF)
        _check(L.mcgen_open(data_root.encode(), version.encode(), C.byref(h), err, ERR_BUF), "mcgen_open", err)
        return cls(h, data_root, version)

    def close(self):
        if self._h:
            load().mcgen_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def dimensions(self) -> list[str]:
        L = load()
        return [L.mcgen_dimension_name(self._h, i).decode() for i in range(L.mcgen_dimension_count(self._h))]

    def presets(self, dimension: str) -> list[str]:
        L = load()
        d = dimension.encode()
        return [L.mcgen_preset_name(self._h, d, i).decode() for i in range(L.mcgen_preset_count(self._h, d))]

    def biome_names(self) -> list[str]:
        L = load()
        return [L.mcgen_biome_name(self._h, i).decode() for i in range(L.mcgen_biome_count(self._h))]

    def world(self, dimension: str = "minecraft:overworld", preset: str = "normal", seeds=0) -> "World":
        return World.create(self, dimension, preset, seeds)

    def selftest(self, npoints: int = 384) -> str:
        buf = C.create_string_buffer(8192)
        _check(load().mcgen_gpu_selftest(self._h, npoints, buf, 8192), "mcgen_gpu_selftest")
        return buf.value.decode()


def _norm_seeds(seeds) -> McSeeds:
    if isinstance(seeds, McSeeds):
        return seeds
    if isinstance(seeds, (tuple, list)):
        return McSeeds(*[int(s) for s in seeds])
    s = int(seeds)
    return McSeeds(s, s, s, s)


SEEDS_LIST, SEEDS_STRUCTURE, SEEDS_RANGE = 0, 1, 2
OBS_BLOCK = 0x100
# one search observation (McGb300Obs): quart or block cell, flags (OBS_BLOCK | End window half-width), mask
OBS_DTYPE = np.dtype([("qx", "<i4"), ("qy", "<i4"), ("qz", "<i4"), ("flags", "<i4"), ("mask", "<u8", (2,))])


def make_obs(rows, block: bool = False, rad: int = 12) -> np.ndarray:
    """Observations from (x, y, z, [biome ids]) rows."""
    a = np.zeros(len(rows), OBS_DTYPE)
    for i, (x, y, z, ids) in enumerate(rows):
        a[i]["qx"], a[i]["qy"], a[i]["qz"] = x, y, z
        a[i]["flags"] = (OBS_BLOCK if block else 0) | rad
        for b in ids:
            a[i]["mask"][b >> 6] |= np.uint64(1) << np.uint64(b & 63)
    return a


class World:
    """McWorld: dimension + preset + seeds."""

    def __init__(self, handle, gen: Generator, dimension: str, preset: str, seeds: McSeeds):
        self._h = handle
        self.gen = gen
        self.dimension = dimension
        self.preset = preset
        self.seeds = seeds

    @classmethod
    def create(cls, gen: Generator, dimension: str, preset: str, seeds) -> "World":
        L = load()
        sd = _norm_seeds(seeds)
        h = _P()
        err = C.create_string_buffer(ERR_BUF)
        _check(L.mcgen_world_new(gen._h, dimension.encode(), preset.encode() if preset else None, C.byref(sd), None, 0,
                                 C.byref(h), err, ERR_BUF), "mcgen_world_new", err)
        return cls(h, gen, dimension, preset, sd)

    def close(self):
        if self._h:
            load().mcgen_world_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def min_y(self) -> int:
        return load().mcgen_world_min_y(self._h)

    @property
    def height(self) -> int:
        return load().mcgen_world_height(self._h)

    @property
    def sea_level(self) -> int:
        return load().mcgen_world_sea_level(self._h)

    # ---- libmcgen biome calls ----
    def biome_at(self, x: int, y: int, z: int) -> int:
        return load().mcgen_biome_at(self._h, int(x), int(y), int(z))

    def biome_grid(self, x0: int, z0: int, nx: int, nz: int, step: int = 1, y: int = 63) -> np.ndarray:
        out = np.empty((nz, nx), np.uint8)
        _check(load().mcgen_biome_grid(self._h, int(x0), int(z0), int(nx), int(nz), int(step), int(y), _ptr(out)),
               "mcgen_biome_grid")
        return out

    def biome_points(self, xyz) -> np.ndarray:
        xyz = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
        out = np.empty(len(xyz), np.uint8)
        ncpu = C.c_int()
        _check(load().mcgen_gpu_biome_points(self._h, len(xyz), _ptr(xyz), _ptr(out), C.byref(ncpu)),
               "mcgen_gpu_biome_points")
        return out

    # ---- additions (mcgen_gb300.h) ----
    def quart_grid(self, qx0: int, qz0: int, nx: int, nz: int, qy: int, tie_rule: int = TIE_ENGINE) -> np.ndarray:
        out = np.empty((nz, nx), np.uint8)
        _check(load().mcgen_gb300_quart_grid(self._h, qx0, qz0, nx, nz, qy, tie_rule, _ptr(out)),
               "mcgen_gb300_quart_grid")
        return out

    def density(self, seed: int, xyz) -> np.ndarray:
        """Overworld density functions at block points: [n, 5] continents, erosion, ridges, offset, depth."""
        xyz = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
        out = np.empty((len(xyz), 5), np.float64)
        _check(load().mcgen_gb300_density_values(self._h, int(seed), len(xyz), _ptr(xyz), _ptr(out)),
               "mcgen_gb300_density_values")
        return out

    def seed_points(self, seeds, qxyz, want_targets: bool = False):
        seeds = np.ascontiguousarray(seeds, dtype=np.int64)
        qxyz = np.ascontiguousarray(qxyz, dtype=np.int32).reshape(-1, 3)
        out = np.empty((len(seeds), len(qxyz)), np.uint8)
        tg = np.empty((len(seeds), len(qxyz), 6), np.int32) if want_targets else None
        _check(load().mcgen_gb300_seed_points(self._h, _ptr(seeds), len(seeds), _ptr(qxyz), len(qxyz), _ptr(out),
                                              _ptr(tg) if tg is not None else None), "mcgen_gb300_seed_points")
        return (out, tg) if want_targets else out

    def search(self, obs: np.ndarray, kind: int = None, base: int = 0, n: int = 0, seeds=None, ties: bool = True,
               max_found: int = 1 << 16):
        """Biome seed search (mcgen_gb300_search): (found seeds sorted as unsigned, reached[nobs + 1], device ms).
        obs: an OBS_DTYPE array; kind: SEEDS_LIST (seeds), SEEDS_STRUCTURE (base, 2^16 candidates) or
        SEEDS_RANGE (base + i, i < n)."""
        obs = np.ascontiguousarray(obs, OBS_DTYPE)
        if kind is None:
            kind = SEEDS_LIST if seeds is not None else SEEDS_STRUCTURE
        lst = None
        if kind == SEEDS_LIST:
            lst = np.ascontiguousarray(seeds, np.int64)
            n = lst.size
        reached = np.zeros(len(obs) + 1, np.uint64)
        found = np.zeros(max(1, max_found), np.int64)
        nf, ms = C.c_uint32(), C.c_double()
        _check(load().mcgen_gb300_search(self._h, kind, _ptr(lst) if lst is not None else None,
                                         C.c_uint64(base & (2**64 - 1)), C.c_uint64(n), obs.ctypes.data, len(obs),
                                         int(ties), _ptr(found), max_found, C.byref(nf), reached.ctypes.data,
                                         C.byref(ms)), "mcgen_gb300_search")
        return found[:nf.value].copy(), reached, ms.value

    def end_radius(self, mask) -> int:
        m = np.ascontiguousarray(mask, np.uint64)
        return load().mcgen_gb300_obs_end_radius(self._h, m.ctypes.data)

    # device-pointer forms: integer addresses of device buffers and a cudaStream_t handle
    def seed_points_dev(self, d_seeds: int, ns: int, d_qxyz: int, np_: int, d_out: int, d_targets: int = 0,
                        stream: int = 0):
        _check(load().mcgen_gb300_seed_points_dev(self._h, d_seeds, ns, d_qxyz, np_, d_out, d_targets or None,
                                                  stream or None), "mcgen_gb300_seed_points_dev")

    def biome_grid_dev(self, x0, z0, nx, nz, step, y, d_out: int, stream: int = 0):
        _check(load().mcgen_gb300_biome_grid_dev(self._h, x0, z0, nx, nz, step, y, d_out, stream or None),
               "mcgen_gb300_biome_grid_dev")

    def quart_grid_seed_dev(self, seed, qx0, qz0, nx, nz, qy, tie_rule, d_out: int, stream: int = 0):
        _check(load().mcgen_gb300_quart_grid_seed_dev(self._h, int(seed), qx0, qz0, nx, nz, qy, tie_rule, d_out,
                                                      stream or None), "mcgen_gb300_quart_grid_seed_dev")

    def quart_grid_dev(self, qx0, qz0, nx, nz, qy, tie_rule, d_out: int, stream: int = 0):
        _check(load().mcgen_gb300_quart_grid_dev(self._h, qx0, qz0, nx, nz, qy, tie_rule, d_out, stream or None),
               "mcgen_gb300_quart_grid_dev")


class RequestArray:
    """Requests as one McGb300Request record array: `worlds` (one World or a sequence, one per request),
    seeds and corners as arrays.  The records hold the worlds' handles; the object keeps the worlds alive."""

    def __init__(self, worlds, seeds, qx0, qz0, nx, nz, qy=16):
        seeds = np.asarray(seeds)
        n = len(seeds)
        rec = np.zeros(n, REQUEST_DTYPE)
        if isinstance(worlds, World):
            self.worlds = [worlds]
            rec["world"] = _handle_int(worlds)
        else:
            self.worlds = list(worlds)
            if len(self.worlds) != n:
                raise ValueError("one world per request")
            rec["world"] = np.array([_handle_int(w) for w in self.worlds], np.uint64)
        rec["seed"] = seeds.astype(np.uint64).view(np.int64) if seeds.dtype == np.uint64 else seeds.astype(np.int64)
        for name, v in (("qx0", qx0), ("qz0", qz0), ("nx", nx), ("nz", nz), ("qy", qy)):
            v = np.broadcast_to(np.asarray(v, np.int64), (n,))
            if v.size and (v.min() < -2**31 or v.max() >= 2**31):
                raise ValueError(f"{name} out of int32 range")
            rec[name] = v
        self.records = rec

    def __len__(self):
        return len(self.records)

    @classmethod
    def from_index(cls, worlds, world_index, seeds, qx0, qz0, nx, nz, qy=16) -> "RequestArray":
        """Requests whose world is worlds[world_index[i]] (a few worlds, many requests)."""
        handles = np.array([_handle_int(w) for w in worlds], np.uint64)
        ra = cls(worlds[0], seeds, qx0, qz0, nx, nz, qy)
        ra.worlds = list(worlds)
        ra.records["world"] = handles[np.asarray(world_index, np.int64)]
        return ra


def _handle_int(w) -> int:
    """A world's McWorld* as an integer (0 for a closed world, which the library rejects with E_ARG)."""
    h = w.handle
    return (h.value or 0) if h is not None else 0


def _pack_requests(requests):
    """[(world, seed, qx0, qz0, nx, nz, qy), ...] -> (record array, worlds)."""
    n = len(requests)
    rec = np.zeros(n, REQUEST_DTYPE)
    if n == 0:
        return rec, []
    cols = list(zip(*requests))
    if len(cols) != 7:
        raise ValueError("a request is (world, seed, qx0, qz0, nx, nz, qy)")
    worlds = list(cols[0])
    handles = {}
    for w in worlds:
        if id(w) not in handles:
            handles[id(w)] = _handle_int(w)
    rec["world"] = np.fromiter((handles[id(w)] for w in worlds), np.uint64, n)
    try:
        rec["seed"] = np.array(cols[1], np.int64)
    except OverflowError:  # seeds given as unsigned 64-bit values
        rec["seed"] = np.fromiter((int(v) & 0xFFFFFFFFFFFFFFFF for v in cols[1]), np.uint64, n).view(np.int64)
    for j, name in enumerate(("qx0", "qz0", "nx", "nz", "qy")):
        v = np.array(cols[2 + j], np.int64)
        if v.min() < -2**31 or v.max() >= 2**31:
            raise ValueError(f"{name} out of int32 range")
        rec[name] = v
    return rec, worlds


class Plan:
    """A frozen batch of quart-grid requests (mcgen_gb300_plan_*): [(world, seed, qx0, qz0, nx, nz, qy), ...]."""

    def __init__(self, requests, tie_rule: int = TIE_ENGINE):
        L = load()
        if isinstance(requests, RequestArray):
            arr, self._worlds = requests.records, list(requests.worlds)
        else:
            arr, self._worlds = _pack_requests(requests)
        h = _P()
        _check(L.mcgen_gb300_plan_new(arr.ctypes.data if len(arr) else None, len(arr), tie_rule, C.byref(h)),
               "mcgen_gb300_plan_new")
        self._h = h
        self.n = len(arr)
        self._nx, self._nz = arr["nx"].copy(), arr["nz"].copy()

    @property
    def shapes(self):
        """(nx, nz) of every request."""
        return list(zip(self._nx.tolist(), self._nz.tolist()))

    def close(self):
        if self._h:
            load().mcgen_gb300_plan_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def output_bytes(self) -> int:
        return load().mcgen_gb300_plan_output_bytes(self._h)

    def offset(self, i: int) -> int:
        return load().mcgen_gb300_plan_output_offset(self._h, i)

    @property
    def shape(self) -> int:
        return load().mcgen_gb300_plan_shape(self._h)

    @shape.setter
    def shape(self, s: int):
        _check(load().mcgen_gb300_plan_set_shape(self._h, s), "mcgen_gb300_plan_set_shape")

    @property
    def h2d_bytes(self) -> int:
        return load().mcgen_gb300_plan_h2d_bytes(self._h)

    def autotune(self, d_out: int, reps: int = 2) -> float:
        ms = C.c_double()
        _check(load().mcgen_gb300_plan_autotune(self._h, d_out, reps, C.byref(ms)), "mcgen_gb300_plan_autotune")
        return ms.value

    def run_dev(self, d_out: int, stream: int = 0, graph: bool = True):
        f = load().mcgen_gb300_plan_run_dev if graph else load().mcgen_gb300_plan_run_dev_direct
        _check(f(self._h, d_out, stream or None), "mcgen_gb300_plan_run_dev")

    def run(self, out: np.ndarray | None = None) -> np.ndarray:
        out = np.empty(self.output_bytes, np.uint8) if out is None else out
        _check(load().mcgen_gb300_plan_run(self._h, _ptr(out)), "mcgen_gb300_plan_run")
        return out

    def split(self, flat: np.ndarray) -> list:
        """Per-request (nz, nx) views of a flat output."""
        return [flat[self.offset(i):self.offset(i) + nx * nz].reshape(nz, nx) for i, (nx, nz) in enumerate(self.shapes)]


class Server:
    """The served form (mcgen_gb300_server_*): continuous batching with a device noise-state cache."""

    def __init__(self, hbm_budget_bytes: int = 8 << 30, max_inflight: int = 2, max_batch: int = 4096):
        h = _P()
        _check(load().mcgen_gb300_server_new(hbm_budget_bytes, max_inflight, max_batch, C.byref(h)),
               "mcgen_gb300_server_new")
        self._h = h
        self._keep = {}

    def close(self):
        if self._h:
            load().mcgen_gb300_server_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, world: "World", seed: int, qx0: int, qz0: int, nx: int, nz: int, qy: int = 16,
               out: np.ndarray | None = None) -> int:
        out = np.empty((nz, nx), np.uint8) if out is None else out
        req = McGb300Request(world.handle, int(seed), qx0, qz0, nx, nz, qy)
        t = C.c_longlong()
        _check(load().mcgen_gb300_server_submit(self._h, C.byref(req), _ptr(out), C.byref(t)),
               "mcgen_gb300_server_submit")
        self._keep[t.value] = out
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1):
        """(ids, latency in ms) of a ticket."""
        lat = C.c_double()
        _check(load().mcgen_gb300_server_wait(self._h, ticket, timeout_ms, C.byref(lat)), "mcgen_gb300_server_wait")
        return self._keep.pop(ticket), lat.value

    def replay(self, requests: "RequestArray", arrival_s, out: np.ndarray, out_off) -> tuple[np.ndarray, float]:
        """Open-loop replay of an arrival schedule from a native submitter thread: (latency from each
        request's scheduled arrival in ms, elapsed seconds).  Request i's ids go to out[out_off[i]:]."""
        arr = np.ascontiguousarray(arrival_s, np.float64)
        off = np.ascontiguousarray(out_off, np.int64)
        n = len(requests)
        if arr.size != n or off.size != n:
            raise ValueError("one arrival time and one output offset per request")
        lat = np.zeros(n, np.float64)
        el = C.c_double()
        rec = requests.records
        _check(load().mcgen_gb300_server_replay(self._h, rec.ctypes.data_as(_P), _ptr(arr), n, _ptr(out), _ptr(off),
                                                _ptr(lat), C.byref(el)), "mcgen_gb300_server_replay")
        return lat, el.value

    def fail_next(self, code: int) -> None:
        """Testing aid: the next batch fails at its allocation step with `code` (host-side injection)."""
        _check(load().mcgen_gb300_server_fail_next(self._h, code), "mcgen_gb300_server_fail_next")

    def stats(self) -> dict:
        st = McGb300ServerStats()
        _check(load().mcgen_gb300_server_stats(self._h, C.byref(st)), "mcgen_gb300_server_stats")
        d = {n: getattr(st, n) for n, _ in st._fields_ if n != "cache_slots"}
        d["cache_slots"] = list(st.cache_slots)
        return d
