"""GPU parity of the biome seed search (mcgen_gb300_search) against the oracle's restatement: found seeds and
the per-depth histogram reached[] must be identical, for every source kind, quart and block observations,
ties on and off, each dimension and both arithmetic branches; and the reference's known-answer files must
give back their seed."""
import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import oracle as O
from search_cases import example_files, oracle_obs, read_example

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mg():
    m = ge.package()
    m.load()
    if m.device_count() < 1:
        pytest.fail("no CUDA device")
    return m


@pytest.fixture(scope="module")
def gens(mg):
    return {v: mg.Generator.open(ge.data_root(), v) for v in ("26.1", "26.2", "26.3", "26.4-snapshot-2")}


def both(mg_world, or_world, obs, **kw):
    f1, r1, ms = mg_world.search(obs, **kw)
    f2, r2 = or_world.search(obs, **kw)
    return f1, r1, f2, r2


@pytest.mark.parametrize("path", example_files(), ids=lambda p: p.rsplit("_", 1)[1][:-4])
def test_known_answer(gens, path):
    version, dim, seed, rows = read_example(path)
    obs = O.make_obs(rows)
    w = gens[version].world("minecraft:" + dim, "normal", 0)
    found, reached, ms = w.search(obs, kind=1, base=seed & ((1 << 48) - 1))
    assert list(found) == [seed]
    _, exp = O.World(ge.data_root(), version, dim).search(obs, O.SEEDS_STRUCTURE, base=seed & ((1 << 48) - 1))
    assert np.array_equal(reached, exp) and ms > 0


@pytest.mark.parametrize("version", ["26.1", "26.3"])
@pytest.mark.parametrize("block", [False, True])
def test_overworld_structure(gens, version, block):
    seed = -4321987654321 if block else 0x1234_5678_9ABC
    obs = oracle_obs(version, "overworld", seed, 6, block, 7)
    w = gens[version].world("minecraft:overworld", "normal", 0)
    ow = O.World(ge.data_root(), version, "overworld")
    for ties in (True, False):
        f1, r1, f2, r2 = both(w, ow, obs, kind=O.SEEDS_STRUCTURE, base=seed & ((1 << 48) - 1), ties=ties)
        assert np.array_equal(r1, r2), (ties, r1, r2)
        assert np.array_equal(f1, f2)
        assert seed in set(f1.tolist())


@pytest.mark.parametrize("version", ["26.2", "26.4-snapshot-2"])
def test_overworld_range_and_list(gens, version):
    seed = 987654321
    obs = oracle_obs(version, "overworld", seed, 5, False, 11, spread=2000)
    w = gens[version].world("minecraft:overworld", "normal", 0)
    ow = O.World(ge.data_root(), version, "overworld")
    f1, r1, f2, r2 = both(w, ow, obs, kind=O.SEEDS_RANGE, base=seed - 30000, n=60000)
    assert np.array_equal(r1, r2) and np.array_equal(f1, f2) and seed in set(f1.tolist())
    rng = np.random.default_rng(5)
    lst = np.concatenate([rng.integers(-2**63, 2**63 - 1, 40000, dtype=np.int64), [seed]])
    f1, r1, f2, r2 = both(w, ow, obs, kind=O.SEEDS_LIST, seeds=lst)
    assert np.array_equal(r1, r2) and np.array_equal(f1, f2) and seed in set(f1.tolist())


@pytest.mark.parametrize("version", ["26.1", "26.3"])
@pytest.mark.parametrize("dim", ["the_nether", "the_end"])
@pytest.mark.parametrize("block", [False, True])
def test_nether_end_list(gens, version, dim, block):
    """Nether and End biomes depend on the low 48 bits only, so candidates are random seeds plus the true one."""
    seed = 0x0BAD_F00D_1234 if not block else -77777777777
    obs = oracle_obs(version, dim, seed, 8, block, 3, spread=20000)
    rng = np.random.default_rng(9)
    lst = np.concatenate([rng.integers(-2**63, 2**63 - 1, 30000, dtype=np.int64), [seed]])
    w = gens[version].world("minecraft:" + dim, "normal", 0)
    ow = O.World(ge.data_root(), version, dim)
    f1, r1, f2, r2 = both(w, ow, obs, kind=O.SEEDS_LIST, seeds=lst)
    assert np.array_equal(r1, r2), (r1, r2)
    assert np.array_equal(f1, f2)
    assert seed in set(f1.tolist())


def test_max_found_and_arguments(gens, mg):
    """More passing candidates than max_found: max_found of them, sorted as unsigned (which ones is unspecified,
    as in the reference: the first to pass); reached[] still counts all.  Bad arguments are refused."""
    w = gens["26.3"].world("minecraft:the_end", "normal", 0)
    obs = oracle_obs("26.3", "the_end", 42, 2, False, 1)
    f1, r1, _ = w.search(obs, kind=O.SEEDS_STRUCTURE, base=42, max_found=10)
    assert int(r1[-1]) == 65536 and len(f1) == 10
    u = f1.view(np.uint64)
    assert np.all(u[1:] > u[:-1]) and np.all((u & np.uint64((1 << 48) - 1)) == np.uint64(42))
    bad = obs.copy()
    bad["flags"][0] = 13
    with pytest.raises(mg.McError):
        w.search(bad, kind=O.SEEDS_STRUCTURE, base=42)
    with pytest.raises(mg.McError):
        w.search(obs[:0], kind=O.SEEDS_STRUCTURE, base=42)


@pytest.mark.parametrize("preset", ["amplified", "large_biomes"])
def test_overworld_presets(gens, preset):
    seed = 0x7777_1234_5678
    obs = oracle_obs("26.3", "overworld", seed, 6, True, 21, spread=3000, preset=preset)
    rng = np.random.default_rng(13)
    lst = np.concatenate([rng.integers(-2**63, 2**63 - 1, 20000, dtype=np.int64), [seed]])
    w = gens["26.3"].world("minecraft:overworld", preset, 0)
    ow = O.World(ge.data_root(), "26.3", "overworld", preset)
    f1, r1, f2, r2 = both(w, ow, obs, kind=O.SEEDS_LIST, seeds=lst)
    assert np.array_equal(r1, r2) and np.array_equal(f1, f2) and seed in set(f1.tolist())
