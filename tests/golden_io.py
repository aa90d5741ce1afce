"""Readers for the committed golden fixtures (tests/golden/)."""
import json
import os

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
VERSIONS = ["26.1", "26.2", "26.3"]


def tsv_rows(version: str, name: str):
    with open(os.path.join(GOLDEN, "vectors", version, name)) as f:
        return [l.rstrip("\n").split("\t") for l in f if l.strip() and not l.startswith("#")]


def grid_hashes(version: str, mode: str = "point"):
    """(dim, seed, qx0, qz0, n, qy, fnv hex) rows of biome_grid_hashes.tsv for one mode."""
    out = []
    for r in tsv_rows(version, "biome_grid_hashes.tsv"):
        if r[2] == mode:
            out.append((r[0], int(r[1]), int(r[3]), int(r[4]), int(r[5]), int(r[6]), r[7]))
    return out


def misc(version: str, cmd: str):
    with open(os.path.join(GOLDEN, "vectors", version, "misc.jsonl")) as f:
        return [d for d in (json.loads(l) for l in f) if d.get("cmd") == cmd]


def refpoint_files():
    d = os.path.join(GOLDEN, "refpoints")
    return sorted(os.path.join(d, f) for f in os.listdir(d) if f.endswith(".npz"))


def parse_refpoint_name(path: str):
    """refpoints_<V>_<dim>_<preset>.npz -> (version, dim, preset)"""
    base = os.path.basename(path)[len("refpoints_"):-len(".npz")]
    preset = base.rsplit("_", 1)[1] if not base.endswith("large_biomes") else "large_biomes"
    rest = base[: -len(preset) - 1]
    for dim in ("overworld", "the_nether", "the_end"):
        if rest.endswith("_" + dim):
            return rest[: -len(dim) - 1], dim, preset
    raise ValueError(path)
