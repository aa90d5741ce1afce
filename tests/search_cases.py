"""Seed-search cases shared by the CPU pins and the GPU parity tests: the reference's known-answer
observation files, and observation sets generated from the oracle at a known seed."""
from __future__ import annotations

import os
import re

import numpy as np

import __graft_entry__ as ge
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
SEARCH_DIR = os.path.join(HERE, "golden", "search")


def example_files():
    return sorted(os.path.join(SEARCH_DIR, f) for f in os.listdir(SEARCH_DIR) if f.startswith("example_obs_"))


def read_example(path):
    """(version, dimension, seed, rows) of a reference example file: 'qx qy qz biome[|biome...]' lines."""
    m = re.search(r"example_obs_([0-9.]+)_(\w+?)_seed(-?\d+)\.txt$", path)
    rows = []
    for ln in open(path):
        if ln.startswith("#") or not ln.strip():
            continue
        x, y, z, names = ln.split()
        rows.append((int(x), int(y), int(z), [O.lib().or_biome_id(n.encode()) for n in names.split("|")]))
    return m.group(1), m.group(2), int(m.group(3)), rows


def oracle_obs(version: str, dim: str, seed: int, k: int, block: bool, rng_seed: int, spread: int = 5000,
               preset: str = "normal"):
    """k observations of `seed` from the oracle: quart cells (or blocks through the zoom) with their biome."""
    rng = np.random.default_rng(rng_seed)
    w = O.World(ge.data_root(), version, dim, preset)
    rows = []
    for _ in range(k):
        x, z = (int(v) for v in rng.integers(-spread, spread, 2))
        y = int(rng.integers(-16, 80)) if dim == "overworld" else 16
        if block:
            b = w.block_points(seed, np.array([[x, y, z]], np.int32))[0]
        else:
            b = w.points(np.array([seed], np.int64), np.array([[x, y, z]], np.int32))[0, 0]
        rows.append((x, y, z, [int(b)]))
    obs = O.make_obs(rows, block=block)
    if dim == "the_end":
        for o in obs:
            o["flags"] = (o["flags"] & O.OBS_BLOCK) | w.end_radius(o["mask"])
    return obs
