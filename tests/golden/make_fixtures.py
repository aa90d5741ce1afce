"""Generate the committed golden fixtures under tests/golden/ (run in the build container).

Sources (read-only, present only where the reference tree is mounted):

* the reference's own golden vectors, produced by its Java oracle on real game code:
  ``tests/vectors/<V>/{climate_overworld,climate_the_nether,climate_the_end,biome_grid_hashes,df}.tsv``,
  the biome-path rows of ``noise.tsv`` and ``misc.jsonl`` (``hashed`` and ``blockbiome`` commands),
  and ``tests/unit/ref26{2,3}.txt`` (NormalNoise bit tables);
* the reference engine's CPU path (``engine/cuda/mcg_host.c``) compiled from its own sources by
  ``oracle/build.py`` -- random seeds x random quart points for every version, dimension and
  Overworld preset, stored as ``refpoints_<V>_<dim>_<preset>.npz`` (seeds, points, biome ids,
  quantised targets).  These extend the pinned cases to presets and 26.4 that the Java vectors lack.
* the reference's seed-search known-answer observation files
  (``crack/src/gpu_biomes/results/example_obs_26.3_overworld_seed*.txt``: quart cells and biomes from its
  Java oracle for a known seed), copied to ``search/``.

Usage:  python tests/golden/make_fixtures.py
"""
from __future__ import annotations

import ctypes as C
import json
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("MCGEN_REFERENCE_ROOT", "/root/reference")  # the reference source tree
VERSIONS = ["26.1", "26.2", "26.3"]
BIOME_NOISES = {"minecraft:offset", "minecraft:temperature", "minecraft:vegetation", "minecraft:continentalness",
                "minecraft:erosion", "minecraft:ridge", "minecraft:nether/temperature",
                "minecraft:nether/vegetation"}


def copy_vectors() -> None:
    for v in VERSIONS:
        src = os.path.join(REF, "tests", "vectors", v)
        dst = os.path.join(HERE, "vectors", v)
        os.makedirs(dst, exist_ok=True)
        for f in ("climate_overworld.tsv", "climate_the_nether.tsv", "climate_the_end.tsv",
                  "biome_grid_hashes.tsv", "df.tsv"):
            shutil.copyfile(os.path.join(src, f), os.path.join(dst, f))
        with open(os.path.join(src, "noise.tsv")) as fi, open(os.path.join(dst, "noise.tsv"), "w") as fo:
            for line in fi:
                if line.startswith("#"):
                    fo.write(line)
                    continue
                r = line.split("\t")
                # overworld noises in the Overworld; the Nether's two legacy biome noises
                if (r[0] == "overworld" and r[2] in BIOME_NOISES) or (r[0] == "the_nether" and r[2].startswith("minecraft:nether/")):
                    fo.write(line)
        with open(os.path.join(src, "misc.jsonl")) as fi, open(os.path.join(dst, "misc.jsonl"), "w") as fo:
            for line in fi:
                if json.loads(line).get("cmd") in ("hashed", "blockbiome"):
                    fo.write(line)
    os.makedirs(os.path.join(HERE, "unit"), exist_ok=True)
    for f in ("ref262.txt", "ref263.txt"):
        shutil.copyfile(os.path.join(REF, "tests", "unit", f), os.path.join(HERE, "unit", f))


def reference_points() -> None:
    sys.path.insert(0, REPO)
    from oracle import build as ob

    path = ob.build_reference()
    if path is None:
        raise SystemExit("reference tree not mounted")
    os.environ["MCGEN_ROOT"] = REF
    L = C.CDLL(path)
    L.ref_open.restype = C.c_void_p
    L.ref_open.argtypes = [C.c_int, C.c_int, C.c_char_p]
    L.ref_close.argtypes = [C.c_void_p]
    L.ref_points.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    rng = np.random.default_rng(20261203)
    outdir = os.path.join(HERE, "refpoints")
    os.makedirs(outdir, exist_ok=True)
    vidx = {"26.1": 0, "26.2": 1, "26.3": 2, "26.4-snapshot-2": 3}
    for v, vi in vidx.items():
        for dim, dname in ((0, "overworld"), (1, "the_nether"), (2, "the_end")):
            for preset in (("normal", "amplified", "large_biomes") if dim == 0 else ("normal",)):
                seeds = rng.integers(-2**63, 2**63 - 1, size=16, dtype=np.int64)
                seeds[:6] = [0, 1, -1, 12345, 2**63 - 1, -2**63]
                pts = []
                for s in (64, 3000, 120000, 7_000_000):
                    pts.append(np.stack([rng.integers(-s, s, 64), rng.integers(-16, 80, 64),
                                         rng.integers(-s, s, 64)], 1))
                pts = np.concatenate(pts).astype(np.int32)
                h = L.ref_open(vi, dim, preset.encode())
                if not h:
                    raise SystemExit(f"reference load failed {v} {dname} {preset}")
                biome = np.zeros((len(seeds), len(pts)), np.uint8)
                tg = np.zeros((len(seeds), len(pts), 6), np.int32)
                L.ref_points(h, seeds.ctypes.data, len(seeds), pts.ctypes.data, len(pts), biome.ctypes.data,
                             tg.ctypes.data)
                L.ref_close(h)
                np.savez_compressed(os.path.join(outdir, f"refpoints_{v}_{dname}_{preset}.npz"), seeds=seeds,
                                    pts=pts, biome=biome, targets=tg)


def copy_search_examples() -> None:
    src = os.path.join(REF, "crack", "src", "gpu_biomes", "results")
    dst = os.path.join(HERE, "search")
    os.makedirs(dst, exist_ok=True)
    for f in sorted(os.listdir(src)):
        if f.startswith("example_obs_") and f.endswith(".txt"):
            shutil.copyfile(os.path.join(src, f), os.path.join(dst, f))


if __name__ == "__main__":
    copy_search_examples()
    copy_vectors()
    reference_points()
    print("fixtures written under", HERE)
