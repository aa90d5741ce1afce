"""Pin the CPU oracle against the reference's golden vectors (CPU only).

Every GPU parity test compares against the oracle, so the oracle is itself checked first against
every fixture the reference holds for this path (tests/golden/, generated by make_fixtures.py).
"""
import struct

import numpy as np
import pytest

from golden_io import VERSIONS, grid_hashes, misc, parse_refpoint_name, refpoint_files, tsv_rows
from oracle import oracle as O

NAMES = None


def names():
    global NAMES
    if NAMES is None:
        NAMES = ["minecraft:" + n for n in O.biome_names()]
    return NAMES


def fbits(x: float) -> int:
    return struct.unpack("<i", struct.pack("<f", x))[0]


def dbits(x: float) -> int:
    return struct.unpack("<q", struct.pack("<d", x))[0]


@pytest.mark.parametrize("version", VERSIONS)
@pytest.mark.parametrize("dim", ["overworld", "the_nether"])
def test_climate_rows(data_root, version, dim):
    """All 6 quantised climate values exact; biome exact, or a fitness tie (Java's thread-local
    lastResult picks among equal leaves; climate_*.tsv rows are single-point queries)."""
    w = O.World(data_root, version, dim)
    rows = tsv_rows(version, f"climate_{dim}.tsv")
    assert len(rows) == 5120
    ties = 0
    for r in rows:
        seed, qx, qy, qz = map(int, r[:4])
        _, tg = w.cell_climate(seed, qx, qy, qz)
        assert list(tg) == [int(x) for x in r[4:10]], r
        leaf, _, nmin = w.tree_find(tg)
        if names()[w.leaf_biome(leaf)] != r[10]:
            assert nmin >= 2, r
            ties += 1
    assert ties <= 2


@pytest.mark.parametrize("version", VERSIONS)
def test_end_rows(data_root, version):
    """End biome per quart and the erosion (height) value bits at the chunk's weird block."""
    w = O.World(data_root, version, "the_end")
    for r in tsv_rows(version, "climate_the_end.tsv"):
        seed, qx, qy, qz = map(int, r[:4])
        assert names()[w.quart_grid(seed, qx, qz, 1, 1, qy)[0, 0]] == r[6]
        cx, cz = (qx * 4) >> 4, (qz * 4) >> 4
        if cx * cx + cz * cz > 4096:
            raw, _ = w.cell_climate(seed, (cx * 2 + 1) * 2, qy, (cz * 2 + 1) * 2)
            assert fbits(float(raw[0])) == int(r[5]), r


NOISE_IDX = {"minecraft:offset": 0, "minecraft:temperature": 1, "minecraft:vegetation": 2,
             "minecraft:continentalness": 3, "minecraft:erosion": 4, "minecraft:ridge": 5,
             "minecraft:nether/temperature": 6, "minecraft:nether/vegetation": 7}


@pytest.mark.parametrize("version", VERSIONS)
def test_noise_rows(data_root, version):
    """NormalNoise values (double bits) of the six climate noises and the two Nether biome noises."""
    ow, ne = O.World(data_root, version, "overworld"), O.World(data_root, version, "the_nether")
    n = 0
    for r in tsv_rows(version, "noise.tsv"):
        w = ow if r[0] == "overworld" else ne
        v = w.noise(int(r[1]), NOISE_IDX[r[2]], float(r[3]), float(r[4]), float(r[5]))
        assert dbits(v) == int(r[7]), r
        n += 1
    assert n == 400


DF_COLUMN = {"minecraft:overworld/continents": 0, "minecraft:overworld/erosion": 1, "minecraft:overworld/ridges": 2,
             "minecraft:overworld/offset": 3, "minecraft:overworld/depth": 4}


def df_rows(version):
    """df.tsv rows grouped by seed: {seed: [(column, x, y, z, dbits, fbits)]}."""
    out = {}
    for r in tsv_rows(version, "df.tsv"):
        out.setdefault(int(r[1]), []).append((DF_COLUMN[r[2]], int(r[3]), int(r[4]), int(r[5]), int(r[7]), int(r[8])))
    return out


@pytest.mark.parametrize("version", VERSIONS)
def test_density_function_bits(data_root, version):
    """df.tsv: continents, erosion, ridges, offset and depth at block points (the reference Java oracle's
    density functions, oracle/gen_vectors.py:76-84), double and float bits exact: the full-precision values
    behind the quantised climate rows (the spline and depth outputs included)."""
    w = O.World(data_root, version, "overworld")
    n = 0
    for seed, rows in df_rows(version).items():
        got = w.density(seed, [(x, y, z) for _, x, y, z, _, _ in rows])
        for (col, x, y, z, db, fb), v in zip(rows, got):
            assert dbits(v[col]) == db, (seed, col, x, y, z)
            assert fbits(v[col]) == fb, (seed, col, x, y, z)
            n += 1
    assert n == 200


@pytest.mark.parametrize("version,fname", [("26.3", "ref263.txt"), ("26.1", "ref262.txt")])
def test_unit_noise_bits(data_root, golden_dir, version, fname):
    """tests/unit/ref26x.txt: NormalNoise bits at raw-double coordinates (float bits for 26.3)."""
    w = O.World(data_root, version, "overworld")
    idx = {"offset": 0, "temperature": 1, "vegetation": 2, "continentalness": 3, "erosion": 4, "ridge": 5}
    n = 0
    with open(f"{golden_dir}/unit/{fname}") as f:
        for line in f:
            p = line.split()
            x, y, z = (struct.unpack("<d", struct.pack("<q", int(t)))[0] for t in p[2:5])
            v = w.noise(int(p[0]), idx[p[1]], x, y, z)
            got = fbits(v) & 0xFFFFFFFF if version == "26.3" else dbits(v) & 0xFFFFFFFFFFFFFFFF
            assert got == int(p[5], 16), line
            n += 1
    assert n == 2160


@pytest.mark.parametrize("version", VERSIONS)
def test_hashed_and_blockbiome(data_root, version):
    for d in misc(version, "hashed"):
        assert O.hashed_seed(d["seed"]) == d["hashed_seed"]
    rows = misc(version, "blockbiome")
    assert len(rows) == 30
    for d in rows:
        w = O.World(data_root, version, d["dim"], d.get("preset", "normal"))
        assert names()[w.biome_at(d["seed"], d["x"], d["y"], d["z"])] == d["biome"], d


@pytest.mark.parametrize("version", VERSIONS)
def test_grid_hash_seed12345(data_root, version):
    """GRID_CHAIN quart grids 1024^2 (End 512^2) at qy=16 reproduce the golden FNV-1a64 digests.
    (All 54 digests are checked on the GPU path; the CPU suite checks seed 12345 of each dimension.)"""
    for dim, seed, qx0, qz0, n, qy, h in grid_hashes(version):
        if seed != 12345:
            continue
        w = O.World(data_root, version, dim)
        g = w.quart_grid(seed, qx0, qz0, n, n, qy, O.TIE_GRID_CHAIN)
        assert O.fnv1a64_names(g) == h, (version, dim)


@pytest.mark.parametrize("path", refpoint_files(), ids=lambda p: p.rsplit("/", 1)[1][10:-4])
def test_reference_engine_points(data_root, path):
    """Random seeds x points (up to +-7M quarts) from the reference engine's CPU path, every
    version, dimension and Overworld preset: biome ids and quantised targets bit-exact."""
    version, dim, preset = parse_refpoint_name(path)
    z = np.load(path)
    w = O.World(data_root, version, dim, preset)
    b, tg = w.points(z["seeds"], z["pts"], want_targets=True)
    assert np.array_equal(b, z["biome"])
    assert np.array_equal(tg, z["targets"])


def test_tree_sizes(data_root):
    assert O.World(data_root, "26.3", "overworld").tree_leaves == 7594
    assert O.World(data_root, "26.1", "overworld").tree_leaves == 7593
    assert O.World(data_root, "26.3", "the_nether").tree_leaves == 5


def test_world_errors(data_root):
    with pytest.raises(RuntimeError):
        O.World(data_root, "25.9", "overworld")
    with pytest.raises(RuntimeError):
        O.World(data_root, "26.3", "overworld", "no_such_preset")
    with pytest.raises(RuntimeError):
        O.World("/nonexistent", "26.3", "overworld")


def test_chunk_mode_grid_hashes(data_root):
    """26.3 "chunk" mode: all six golden FNV-1a64 digests of the 1024^2 Overworld grids whose ties are chained
    in chunk order (the Java oracle's chunk-batched climate), pinned by the oracle's chunk-order grid."""
    rows = grid_hashes("26.3", "chunk")
    assert len(rows) == 6
    w = O.World(data_root, "26.3", "overworld")
    for dim, seed, qx0, qz0, n, qy, h in rows:
        assert O.fnv1a64_names(w.chunk_order_grid(seed, qx0, qz0, n, n, qy)) == h, seed
