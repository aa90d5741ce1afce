"""GPU parity: the sm_103a kernels, called through the C ABI, against the oracle and the golden fixtures.

Bit-exact for every id and quantised target.  Cases follow the reference's own tests: the Java-oracle
golden vectors (climate rows, FNV grid digests, zoom rows), the reference engine's random seed x point
tables (every version, dimension and Overworld preset), and the reference GPU test's method of many
seeds x points at growing coordinate scales (crack/src/gpu_biomes/test_gpu_biomes.cu:18,56-75).
"""
import numpy as np
import pytest

import __graft_entry__ as ge
from golden_io import VERSIONS, grid_hashes, misc, parse_refpoint_name, refpoint_files, tsv_rows
from oracle import oracle as O

pytestmark = pytest.mark.gpu
ALL_VERSIONS = VERSIONS + ["26.4-snapshot-2"]


@pytest.fixture(scope="module")
def mg():
    m = ge.package()
    m.load()
    if m.device_count() < 1:
        pytest.fail("no CUDA device: the GPU tests need one (there is no CPU path)")
    return m


@pytest.fixture(scope="module")
def gens(mg):
    return {v: mg.Generator.open(ge.data_root(), v) for v in ALL_VERSIONS}


NAMES = ["minecraft:" + n for n in O.biome_names()]


@pytest.mark.parametrize("path", refpoint_files(), ids=lambda p: p.rsplit("/", 1)[1][10:-4])
def test_reference_engine_points(gens, path):
    """Seeds x quart points from the reference engine's own CPU path: biome ids and targets."""
    version, dim, preset = parse_refpoint_name(path)
    z = np.load(path)
    w = gens[version].world("minecraft:" + dim, preset, 0)
    b, tg = w.seed_points(z["seeds"], z["pts"], want_targets=True)
    assert np.array_equal(b, z["biome"]), int((b != z["biome"]).sum())
    if dim != "the_end":
        assert np.array_equal(tg, z["targets"])


@pytest.mark.parametrize("version", VERSIONS)
@pytest.mark.parametrize("dim", ["overworld", "the_nether", "the_end"])
def test_golden_climate_rows(gens, version, dim):
    """Java-oracle climate rows: 6 targets exact; biome exact or an R-tree fitness tie."""
    rows = tsv_rows(version, f"climate_{dim}.tsv")
    w = gens[version].world("minecraft:" + dim, "normal", 0)
    ow = O.World(ge.data_root(), version, dim)
    by_seed = {}
    for r in rows:
        by_seed.setdefault(int(r[0]), []).append(r)
    mism = 0
    for seed, rs in by_seed.items():
        pts = np.array([[int(r[1]), int(r[2]), int(r[3])] for r in rs], np.int32)
        b, tg = w.seed_points(np.array([seed], np.int64), pts, want_targets=True)
        for i, r in enumerate(rs):
            name = r[6] if dim == "the_end" else r[10]
            if dim != "the_end":
                assert list(tg[0, i]) == [int(x) for x in r[4:10]], r
            if NAMES[b[0, i]] != name:
                _, _, nmin = ow.tree_find(tg[0, i].astype(np.int64))
                assert dim != "the_end" and nmin >= 2, r
                mism += 1
    assert mism <= 2


@pytest.mark.parametrize("version", VERSIONS)
def test_golden_grid_hashes(gens, version):
    """All FNV-1a64 digests of the golden 1024^2 (End 512^2) quart grids, GRID_CHAIN tie rule."""
    n = 0
    for dim, seed, qx0, qz0, size, qy, h in grid_hashes(version):
        w = gens[version].world("minecraft:" + dim, "normal", seed)
        g = w.quart_grid(qx0, qz0, size, size, qy, ge.package().TIE_GRID_CHAIN)
        assert O.fnv1a64_names(g) == h, (dim, seed)
        n += 1
    assert n == 18


@pytest.mark.parametrize("version", VERSIONS)
def test_golden_blockbiome(gens, version):
    """BiomeManager zoom rows (blockbiome) through mcgen_biome_at."""
    for d in misc(version, "blockbiome"):
        w = gens[version].world("minecraft:" + d["dim"], d.get("preset", "normal"), d["seed"])
        assert NAMES[w.biome_at(d["x"], d["y"], d["z"])] == d["biome"], d



DF_COLUMN = {"minecraft:overworld/continents": 0, "minecraft:overworld/erosion": 1, "minecraft:overworld/ridges": 2,
             "minecraft:overworld/offset": 3, "minecraft:overworld/depth": 4}


@pytest.mark.parametrize("version", VERSIONS)
def test_golden_density_functions(gens, version):
    """df.tsv: continents, erosion, ridges, offset and depth at block points, computed on the device through
    the C ABI (mcgen_gb300_density_values): double and float bits exact, 200 rows per version; and the same
    on random block points against the oracle."""
    import struct
    w = gens[version].world("minecraft:overworld", "normal", 0)
    rows = {}
    for r in tsv_rows(version, "df.tsv"):
        rows.setdefault(int(r[1]), []).append((DF_COLUMN[r[2]], int(r[3]), int(r[4]), int(r[5]), int(r[7]), int(r[8])))
    n = 0
    for seed, rs in rows.items():
        got = w.density(seed, [(x, y, z) for _, x, y, z, _, _ in rs])
        for (col, x, y, z, db, fb), v in zip(rs, got):
            assert struct.unpack("<q", struct.pack("<d", v[col]))[0] == db, (seed, col, x, y, z)
            assert struct.unpack("<i", struct.pack("<f", v[col]))[0] == fb, (seed, col, x, y, z)
            n += 1
    assert n == 200
    rng = np.random.default_rng(31)
    ow = O.World(ge.data_root(), version, "overworld")
    for seed in rng.integers(-2**63, 2**63 - 1, 4, dtype=np.int64):
        xyz = np.stack([rng.integers(-2_000_000, 2_000_000, 512), rng.integers(-80, 340, 512),
                        rng.integers(-2_000_000, 2_000_000, 512)], 1)
        assert np.array_equal(w.density(int(seed), xyz).view(np.int64), ow.density(int(seed), xyz).view(np.int64))

@pytest.mark.parametrize("version", ALL_VERSIONS)
@pytest.mark.parametrize("dim", ["overworld", "the_nether", "the_end"])
def test_biome_grid_dropin(gens, version, dim):
    """mcgen_biome_grid (zoom + chunk-cell ties) against the oracle: step 4 at y=64, a step-1 patch at a
    negative corner, and a sparse large-coordinate grid."""
    for seed, args in ((12345, (-512, -512, 64, 64, 4, 64)), (-7, (-1000, -37, 40, 24, 1, -50)),
                       (2**63 - 1, (-9_000_000, 5_000_000, 16, 16, 1_000_003, 100))):
        w = gens[version].world("minecraft:" + dim, "normal", seed)
        got = w.biome_grid(*args)
        exp = O.World(ge.data_root(), version, dim).biome_grid(seed, *args)
        assert np.array_equal(got, exp), (seed, args, int((got != exp).sum()))


@pytest.mark.parametrize("version", ["26.1", "26.3"])
@pytest.mark.parametrize("preset", ["amplified", "large_biomes"])
def test_biome_grid_presets(gens, version, preset):
    w = gens[version].world("minecraft:overworld", preset, 99)
    got = w.biome_grid(-300, 200, 48, 48, 8, 70)
    exp = O.World(ge.data_root(), version, "overworld", preset).biome_grid(99, -300, 200, 48, 48, 8, 70)
    assert np.array_equal(got, exp)


@pytest.mark.parametrize("version", ALL_VERSIONS)
def test_block_points(gens, version):
    """mcgen_gpu_biome_points at random block points, including world-height extremes (y clamp)."""
    rng = np.random.default_rng(11)
    for dim in ("overworld", "the_nether", "the_end"):
        w = gens[version].world("minecraft:" + dim, "normal", 8675309)
        xyz = np.stack([rng.integers(-200000, 200000, 300), rng.integers(-200, 500, 300),
                        rng.integers(-200000, 200000, 300)], 1).astype(np.int32)
        got = w.biome_points(xyz)
        exp = O.World(ge.data_root(), version, dim).block_points(8675309, xyz)
        assert np.array_equal(got, exp), dim


@pytest.mark.parametrize("version", ["26.1", "26.3"])
@pytest.mark.parametrize("dim", ["overworld", "the_nether", "the_end"])
def test_quart_grid_engine(gens, version, dim):
    w = gens[version].world("minecraft:" + dim, "normal", 4242)
    got = w.quart_grid(-200, 100, 96, 80, 16, ge.package().TIE_ENGINE)
    exp = O.World(ge.data_root(), version, dim).quart_grid(4242, -200, 100, 96, 80, 16, O.TIE_ENGINE)
    assert np.array_equal(got, exp)


@pytest.mark.parametrize("version", ["26.1", "26.3"])
def test_many_seeds_scales(gens, version):
    """The reference GPU test's shape: edge seeds + random seeds x points at four coordinate scales,
    up to +-7.5M quarts (crack/src/gpu_biomes/test_gpu_biomes.cu:18,56-63)."""
    rng = np.random.default_rng(3)
    seeds = np.concatenate([np.array([0, 1, -1, 2**63 - 1, -2**63, 12345, 1 << 32, -(1 << 48), 0x5DEECE66D], np.int64),
                            rng.integers(-2**63, 2**63 - 1, 503, dtype=np.int64)])
    for scale in (64, 4096, 262144, 7_500_000):
        pts = np.stack([rng.integers(-scale, scale, 16), rng.integers(-16, 80, 16), rng.integers(-scale, scale, 16)], 1)
        for dim in ("overworld", "the_nether"):
            w = gens[version].world("minecraft:" + dim, "normal", 0)
            b, tg = w.seed_points(seeds, pts, want_targets=True)
            eb, etg = O.World(ge.data_root(), version, dim).points(seeds, pts, want_targets=True)
            assert np.array_equal(tg, etg), (scale, dim)
            assert np.array_equal(b, eb), (scale, dim)


def test_config1_dropin_full(gens):
    """Overworld 26.3, seed 12345, 256x256 cells x,z in [-512,512) step 4 at y=64: the drop-in form of
    the plain-method workload, bit-exact against the oracle."""
    w = gens["26.3"].world("minecraft:overworld", "normal", 12345)
    got = w.biome_grid(-512, -512, 256, 256, 4, 64)
    exp = O.World(ge.data_root(), "26.3", "overworld").biome_grid(12345, -512, -512, 256, 256, 4, 64)
    assert np.array_equal(got, exp)


def test_config2_shape(gens):
    """65,536 SplitMix64 seeds x 8 points (Overworld 26.3): a 4,096-seed stride sample bit-exact against
    the oracle, and the full batch deterministic across calls."""
    import bench

    seeds, pts = bench.config2_inputs()
    w = gens["26.3"].world("minecraft:overworld", "normal", 0)
    a = w.seed_points(seeds, pts)
    b = w.seed_points(seeds, pts)
    assert np.array_equal(a, b)
    sub = np.arange(0, len(seeds), 16)
    exp = O.World(ge.data_root(), "26.3", "overworld").points(seeds[sub], pts)
    assert np.array_equal(a[sub], exp)


def test_edge_sizes(gens):
    w = gens["26.3"].world("minecraft:overworld", "normal", 1)
    one = w.biome_grid(5, 5, 1, 1, 1, 64)
    assert one.shape == (1, 1) and one[0, 0] == w.biome_at(5, 64, 5)
    assert w.seed_points(np.zeros(0, np.int64), np.zeros((3, 3), np.int32)).shape == (0, 3)
    row = w.quart_grid(0, 0, 1000, 1, 16, 0)
    exp = O.World(ge.data_root(), "26.3", "overworld").quart_grid(1, 0, 0, 1000, 1, 16)
    assert np.array_equal(row, exp)


def test_fast_coordinate_split(mg):
    """The integer coordinate split that replaces seven of the eight FP64 operations of every octave
    coordinate equals the reference's double arithmetic on 2^26 generated inputs per branch."""
    for seed in (1, 2):
        bf, bd = mg.check_split(1 << 26, seed)
        assert (bf, bd) == (0, 0)


def test_fixed_point_octave(mg):
    """The double branch's fixed-point octave (exact gradient sums, once-rounded first lerp differences)
    equals the plain double octave on 2^24 random permutations x fractions."""
    for seed in (3, 4):
        assert mg.check_octave(1 << 24, seed) == 0


def test_end_island_screen(mg):
    """The End's screened island test (float corner terms, exact double only near the -0.9 threshold) on
    2^26 random (permutation, chunk cell) cases of both branches: every decision equals the reference's double
    simplex, the float evaluation stays within its bound, and only a small share needs the exact value."""
    bad, left, worst = mg.check_end(1 << 26, 77)
    assert bad == 0
    assert worst < 1.0
    assert 0 < left < (1 << 26) // 100  # values near the threshold occurred and took the exact value


def test_zoom_screen(mg):
    """BiomeManager's zoom choice, screened in single precision, equals the double-precision first minimum of
    the 8 candidates on 2^27 random (zoom seed, block) cases, and the double-precision fallback ran."""
    for seed in (5, 6):
        bad, screened_out = mg.check_zoom(1 << 27, seed)
        assert bad == 0
        assert screened_out > 0


@pytest.mark.parametrize("version", ["26.1", "26.2"])
@pytest.mark.parametrize("dim", ["minecraft:overworld", "minecraft:the_nether"])
def test_noise_screen(gens, mg, version, dim):
    """The double branch's climate noises evaluated in fixed point and screened by their error bound give the
    exact double path's floats on 2^22 random coordinates per seed; the bound holds with room (the largest
    observed error is a small fraction of it) and the exact path is left only a small share of the values.
    The values left to it are the dangerous ones -- the double value within the bound of a float rounding
    boundary, where the screen must say "unsettled" -- and the test requires that such values occurred (a
    few thousand per seed), each one exact."""
    for seed in (12345, -(2**62) + 17):
        w = gens[version].world(dim, "normal", seed)
        bad, left, worst = mg.check_noise(w, 1 << 22, seed & 0xFFFF)
        n_values = (1 << 22) * (6 if dim.endswith("overworld") else 2)
        print(f"{version} {dim} seed {seed}: worst error / bound {worst:.4f}, left to the exact path {left / n_values:.2e}")
        assert bad == 0
        assert worst < 0.5
        assert 0 < left < n_values // 50


@pytest.mark.parametrize("version", ["26.1", "26.2"])
@pytest.mark.parametrize("dim", ["minecraft:overworld", "minecraft:the_nether"])
def test_noise_quant_screen(gens, mg, version, dim):
    """The 32-bit screen of the double branch's noises whose value is only quantised (the Nether kernels'
    form for their two noises; checked on the Overworld's temperature and vegetation too, whose constants
    differ) gives quantize((float)exact) wherever it settles the target, on 2^22 random coordinates per seed; its error stays well inside the bound, it leaves under 2 % of the values to the 59-bit screen, and
    values whose exact double lies within twice the bound of a target boundary occurred among the settled
    ones (the cases that try the bound)."""
    for seed in (12345, -(2**62) + 17):
        w = gens[version].world(dim, "normal", seed)
        bad, left, worst, near = mg.check_noise_quant(w, 1 << 22, seed & 0xFFFF)
        n_values = (1 << 22) * 2
        print(f"{version} {dim} seed {seed}: worst error / bound {worst:.4f}, left {left / n_values:.2e}, "
              f"near a boundary {near}")
        assert bad == 0
        assert worst < 0.8
        assert 0 < left < n_values // 50
        assert near > 0


@pytest.mark.parametrize("version", ["26.1", "26.2"])
@pytest.mark.parametrize("preset", ["normal", "large_biomes", "amplified"])
def test_climate_screen(gens, mg, version, preset):
    """The double branch's Overworld climate as the kernels compute it (exact shift noises, climate noises
    screened in fixed point) gives the plain double evaluation's six targets on 2^21 random quart cells per
    seed out to |q| = 2^21, and the screen leaves only a small share of the cells to the exact path."""
    for seed in (12345, -(2**62) + 17):
        w = gens[version].world("minecraft:overworld", preset, seed)
        bad, fallback = mg.check_climate(w, 1 << 21, seed & 0xFFFF)
        print(f"{version} {preset} seed {seed}: cells with a value left to the exact path {fallback / (1 << 21):.2e}")
        assert bad == 0
        assert 0 < fallback < (1 << 21) // 10


@pytest.mark.parametrize("version", ["26.1", "26.3", "26.4-snapshot-2"])
@pytest.mark.parametrize("preset", ["normal", "large_biomes", "amplified"])
@pytest.mark.parametrize("dim", ["minecraft:overworld", "minecraft:the_nether"])
def test_tree_search_32bit(gens, mg, version, preset, dim):
    """The level-unrolled and single-loop R-tree searches with 32-bit clamped box distances, and the tie
    search, return the 64-bit stack searches' leaf, fitness and tie flag on 2^20 random targets, half of
    them beyond the clamp (where the 64-bit search takes over)."""
    if dim.endswith("nether") and preset != "normal":
        pytest.skip("the Nether has no presets")
    w = gens[version].world(dim, preset, 1)
    bad_leaf, bad_other = mg.check_tree(w, 1 << 20, 77)
    assert bad_leaf == 0 and bad_other == 0


def test_chunk_mode_grid_hashes(gens, mg):
    """The six golden 26.3 "chunk" digests through mcgen_gb300_quart_grid with MCGEN_TIE_CHUNK_ORDER, and an
    unaligned grid (partial chunks on every side) against the oracle."""
    rows = grid_hashes("26.3", "chunk")
    assert len(rows) == 6
    for dim, seed, qx0, qz0, n, qy, h in rows:
        w = gens["26.3"].world("minecraft:" + dim, "normal", seed)
        assert O.fnv1a64_names(w.quart_grid(qx0, qz0, n, n, qy, mg.TIE_CHUNK_ORDER)) == h, seed
    w = gens["26.3"].world("minecraft:overworld", "normal", 777)
    got = w.quart_grid(-301, 129, 203, 97, 16, mg.TIE_CHUNK_ORDER)
    exp = O.World(ge.data_root(), "26.3", "overworld").chunk_order_grid(777, -301, 129, 203, 97, 16)
    assert np.array_equal(got, exp)


@pytest.mark.parametrize("version,dim", [("26.3", "overworld"), ("26.1", "the_end"), ("26.4-snapshot-2", "the_nether")])
def test_map2048_rows(gens, version, dim):
    """The reference's GPU map benchmark shape (2048 x 2048 cells, x,z from -4096 step 4, y=64, seed 12345):
    the whole map on the GPU, rows at the edges and the middle against the oracle."""
    w = gens[version].world("minecraft:" + dim, "normal", 12345)
    got = w.biome_grid(-4096, -4096, 2048, 2048, 4, 64)
    ow = O.World(ge.data_root(), version, dim)
    for r in (0, 1023, 2047):
        exp = ow.biome_grid(12345, -4096, -4096 + 4 * r, 2048, 1, 4, 64)
        assert np.array_equal(got[r:r + 1], exp), (r, int((got[r:r + 1] != exp).sum()))
