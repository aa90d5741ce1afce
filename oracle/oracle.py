"""ctypes binding of the CPU oracle (test infrastructure only).

Loaded by tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg, which compare the
GPU path's outputs with it.  The product library never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

OVERWORLD, NETHER, END = 0, 1, 2
TIE_ENGINE, TIE_GRID_CHAIN, TIE_CHUNK_CELL = 0, 1, 2
DIMS = {"overworld": OVERWORLD, "minecraft:overworld": OVERWORLD, "the_nether": NETHER, "nether": NETHER,
        "minecraft:the_nether": NETHER, "the_end": END, "end": END, "minecraft:the_end": END}

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        vp, i32, i64, u8p, i32p, i64p = C.c_void_p, C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p
        L.or_world_load.restype = vp
        L.or_world_load.argtypes = [C.c_char_p, C.c_char_p, i32, C.c_char_p, C.c_char_p, C.c_size_t]
        L.or_world_free.argtypes = [vp]
        for f in ("or_world_version", "or_world_float_mode", "or_tree_nodes", "or_tree_leaves"):
            getattr(L, f).argtypes = [vp]
            getattr(L, f).restype = i32
        L.or_biome_count.restype = i32
        L.or_biome_name.restype = C.c_char_p
        L.or_biome_name.argtypes = [i32]
        L.or_biome_id.restype = i32
        L.or_biome_id.argtypes = [C.c_char_p]
        L.or_hashed_seed.restype = i64
        L.or_hashed_seed.argtypes = [i64]
        L.or_noise_value.restype = C.c_double
        L.or_noise_value.argtypes = [vp, i64, i32, C.c_double, C.c_double, C.c_double]
        L.or_points.argtypes = [vp, i64p, i32, i32p, i32, u8p, i32p, i32]
        L.or_quart_grid.argtypes = [vp, i64, i32, i32, i32, i32, i32, i32, u8p, i32]
        L.or_biome_at.restype = i32
        L.or_biome_at.argtypes = [vp, i64, i32, i32, i32]
        L.or_biome_grid.argtypes = [vp, i64, i32, i32, i32, i32, i32, i32, u8p, i32]
        L.or_block_points.argtypes = [vp, i64, i32, i32p, u8p, i32]
        L.or_cell_climate.argtypes = [vp, i64, i32, i32, i32, C.c_void_p, i64p]
        L.or_tree_find.restype = i32
        L.or_tree_find.argtypes = [vp, i64p, C.POINTER(C.c_int64), C.POINTER(C.c_int)]
        L.or_leaf_biome.restype = i32
        L.or_leaf_biome.argtypes = [vp, i32]
        L.or_tree_export.restype = i32
        L.or_tree_export.argtypes = [vp, C.c_void_p, C.c_void_p, C.c_void_p]
        L.or_density.restype = i32
        L.or_density.argtypes = [vp, i64, i32, i32p, C.c_void_p]
        L.or_tree_kids.restype = i32
        L.or_tree_kids.argtypes = [vp]
        L.or_points_work.argtypes = [vp, i64, i32p, i32, C.c_void_p]
        L.or_chunk_grid.argtypes = [vp, i64, i32, i32, i32, i32, i32, u8p, i32]
        L.or_fnv1a64_names.restype = C.c_uint64
        L.or_fnv1a64_names.argtypes = [u8p, C.c_size_t]
        L.or_chunk_order_grid.argtypes = [vp, i64, i32, i32, i32, i32, i32, u8p]
        L.or_search.argtypes = [vp, i32, i64p, C.c_uint64, C.c_uint64, C.c_void_p, i32, i32, C.c_void_p, i64p,
                                C.c_uint32, C.POINTER(C.c_uint32), i32]
        L.or_obs_end_radius.restype = i32
        L.or_obs_end_radius.argtypes = [vp, C.c_void_p]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def biome_names() -> list[str]:
    L = lib()
    return [L.or_biome_name(i).decode() for i in range(L.or_biome_count())]


def biome_id(name: str) -> int:
    return lib().or_biome_id(name.encode())


def hashed_seed(seed: int) -> int:
    return lib().or_hashed_seed(seed)


SEEDS_LIST, SEEDS_STRUCTURE, SEEDS_RANGE = 0, 1, 2
OBS_BLOCK = 0x100
# one observation: qx, qy, qz, flags (OBS_BLOCK | End window half-width), mask[2]
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
    """One (data root, version, dimension, preset) of the oracle."""

    def __init__(self, root: str, version: str, dim, preset: str = "normal"):
        L = lib()
        d = DIMS[dim] if isinstance(dim, str) else int(dim)
        err = C.create_string_buffer(512)
        self._h = L.or_world_load(root.encode(), version.encode(), d, preset.encode(), err, 512)
        if not self._h:
            raise RuntimeError(err.value.decode())
        self.dim = d
        self.version = version

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.or_world_free(h)
            self._h = None

    @property
    def float_mode(self) -> bool:
        return bool(lib().or_world_float_mode(self._h))

    @property
    def tree_leaves(self) -> int:
        return lib().or_tree_leaves(self._h)

    def density(self, seed: int, xyz) -> np.ndarray:
        """Overworld density functions at block points: [n, 5] continents, erosion, ridges, offset, depth."""
        xyz = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
        out = np.zeros((len(xyz), 5), np.float64)
        if lib().or_density(self._h, seed, len(xyz), _ptr(xyz), _ptr(out)) != 0:
            raise ValueError("density functions are defined for the Overworld")
        return out

    def tree(self):
        """The R-tree as built: (root, lo[n,7], hi[n,7], first[n], count[n], biome[n], kids[])."""
        n = lib().or_tree_nodes(self._h)
        lohi = np.zeros((n, 14), np.int64)
        fcb = np.zeros((n, 3), np.int32)
        kids = np.zeros(max(1, lib().or_tree_kids(self._h)), np.int32)
        root = lib().or_tree_export(self._h, _ptr(lohi), _ptr(fcb), _ptr(kids))
        return root, lohi[:, :7], lohi[:, 7:], fcb[:, 0], fcb[:, 1], fcb[:, 2], kids

    def noise(self, seed: int, which: int, x: float, y: float, z: float) -> float:
        return lib().or_noise_value(self._h, seed, which, x, y, z)

    def points(self, seeds, pts, threads: int = 0, want_targets: bool = False):
        seeds = np.ascontiguousarray(seeds, dtype=np.int64)
        pts = np.ascontiguousarray(pts, dtype=np.int32).reshape(-1, 3)
        out = np.zeros((len(seeds), len(pts)), dtype=np.uint8)
        tg = np.zeros((len(seeds), len(pts), 6), dtype=np.int32) if want_targets else None
        lib().or_points(self._h, _ptr(seeds), len(seeds), _ptr(pts), len(pts), _ptr(out),
                        _ptr(tg) if tg is not None else None, threads)
        return (out, tg) if want_targets else out

    def quart_grid(self, seed: int, qx0: int, qz0: int, nx: int, nz: int, qy: int, rule: int = TIE_ENGINE,
                   threads: int = 0) -> np.ndarray:
        out = np.zeros((nz, nx), dtype=np.uint8)
        lib().or_quart_grid(self._h, seed, qx0, qz0, nx, nz, qy, rule, _ptr(out), threads)
        return out

    def chunk_grid(self, seed: int, qx0: int, qz0: int, nx: int, nz: int, qy: int, threads: int = 0) -> np.ndarray:
        out = np.zeros((nz, nx), dtype=np.uint8)
        lib().or_chunk_grid(self._h, seed, qx0, qz0, nx, nz, qy, _ptr(out), threads)
        return out

    def biome_at(self, seed: int, x: int, y: int, z: int) -> int:
        return lib().or_biome_at(self._h, seed, x, y, z)

    def biome_grid(self, seed: int, x0: int, z0: int, nx: int, nz: int, step: int, y: int,
                   threads: int = 0) -> np.ndarray:
        out = np.zeros((nz, nx), dtype=np.uint8)
        lib().or_biome_grid(self._h, seed, x0, z0, nx, nz, step, y, _ptr(out), threads)
        return out

    def block_points(self, seed: int, xyz, threads: int = 0) -> np.ndarray:
        xyz = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
        out = np.zeros(len(xyz), dtype=np.uint8)
        lib().or_block_points(self._h, seed, len(xyz), _ptr(xyz), _ptr(out), threads)
        return out

    def cell_climate(self, seed: int, qx: int, qy: int, qz: int):
        raw = np.zeros(6, dtype=np.float32)
        tg = np.zeros(6, dtype=np.int64)
        lib().or_cell_climate(self._h, seed, qx, qy, qz, _ptr(raw), _ptr(tg))
        return raw, tg

    def tree_find(self, tg6):
        tg = np.ascontiguousarray(tg6, dtype=np.int64)
        d = C.c_int64()
        n = C.c_int()
        leaf = lib().or_tree_find(self._h, _ptr(tg), C.byref(d), C.byref(n))
        return leaf, d.value, n.value

    def leaf_biome(self, leaf: int) -> int:
        return lib().or_leaf_biome(self._h, leaf)

    def chunk_order_grid(self, seed: int, qx0: int, qz0: int, nx: int, nz: int, qy: int) -> np.ndarray:
        """26.3 "chunk" mode grid: ties chained in chunk order across the grid."""
        out = np.empty((nz, nx), np.uint8)
        lib().or_chunk_order_grid(self._h, seed, qx0, qz0, nx, nz, qy, _ptr(out))
        return out

    def search(self, obs: np.ndarray, kind: int = SEEDS_STRUCTURE, base: int = 0, n: int = 0, seeds=None,
               ties: bool = True, max_found: int = 1 << 16, threads: int = 0):
        """Seed search: (found seeds sorted as unsigned, reached[nobs + 1])."""
        obs = np.ascontiguousarray(obs, OBS_DTYPE)
        lst = None
        if kind == SEEDS_LIST:
            lst = np.ascontiguousarray(seeds, np.int64)
            n = lst.size
        reached = np.zeros(len(obs) + 1, np.uint64)
        found = np.zeros(max(1, max_found), np.int64)
        nf = C.c_uint32()
        lib().or_search(self._h, kind, _ptr(lst) if lst is not None else None, C.c_uint64(base & (2**64 - 1)),
                        C.c_uint64(n), obs.ctypes.data, len(obs), int(ties), reached.ctypes.data, _ptr(found),
                        max_found, C.byref(nf), threads)
        return found[:nf.value].copy(), reached

    def end_radius(self, mask) -> int:
        m = np.ascontiguousarray(mask, np.uint64)
        return lib().or_obs_end_radius(self._h, m.ctypes.data)

    def work(self, seed: int, pts):
        pts = np.ascontiguousarray(pts, dtype=np.int32).reshape(-1, 3)
        w = np.zeros(4, dtype=np.int64)
        lib().or_points_work(self._h, seed, _ptr(pts), len(pts), _ptr(w))
        return dict(zip(("octave_samples", "tree_nodes", "tree_queries", "spline_nodes"), w.tolist()))


def fnv1a64_names(ids: np.ndarray) -> str:
    """FNV-1a 64 over 'minecraft:<name>\\n' per cell in array order (biome_grid_hashes.tsv digest)."""
    a = np.ascontiguousarray(ids, dtype=np.uint8).reshape(-1)
    return f"{lib().or_fnv1a64_names(_ptr(a), a.size):016x}"
