"""The batched form (one persistent launch over many uneven requests) against the oracle and against the
plain one-request-per-launch form: bit-exact per request, for every version and dimension mixed in one
batch, both tie rules, graph replays, every tile shape of the autotuner."""
import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import oracle as O

pytestmark = pytest.mark.gpu
VERSIONS = ["26.1", "26.2", "26.3", "26.4-snapshot-2"]
DIMS = ["minecraft:overworld", "minecraft:the_nether", "minecraft:the_end"]


@pytest.fixture(scope="module")
def env():
    mg = ge.package()
    mg.load()
    if mg.device_count() < 1:
        pytest.fail("no CUDA device")
    gens = {v: mg.Generator.open(ge.data_root(), v) for v in VERSIONS}
    worlds = {(v, d): gens[v].world(d, "normal", 0) for v in VERSIONS for d in DIMS}
    return mg, gens, worlds


def mixed_requests(worlds, n=48, seed=9):
    rng = np.random.default_rng(seed)
    keys = list(worlds)
    reqs = []
    shapes = [(1, 1), (1, 37), (37, 1), (33, 5), (64, 64), (17, 129), (130, 3), (48, 48)]
    for i in range(n):
        v, d = keys[i % len(keys)]
        nx, nz = shapes[i % len(shapes)]
        qx0 = int(rng.integers(-9000, 9000)) if i % 5 else -nx // 2  # some straddle the origin (End disc)
        qz0 = int(rng.integers(-9000, 9000)) if i % 5 else -nz // 2
        seed_i = int(rng.integers(-2**63, 2**63 - 1))
        reqs.append(((v, d), seed_i, qx0, qz0, nx, nz, 16))
    return reqs


def oracle_grid(v, d, seed, qx0, qz0, nx, nz, qy, rule):
    w = O.World(ge.data_root(), v, d.split(":")[1])
    if rule == 2 and not d.endswith("the_end"):
        return w.chunk_grid(seed, qx0, qz0, nx, nz, qy)
    return w.quart_grid(seed, qx0, qz0, nx, nz, qy, O.TIE_ENGINE)


@pytest.mark.parametrize("rule", [0, 2])
def test_batch_matches_oracle(env, rule):
    mg, gens, worlds = env
    reqs = mixed_requests(worlds)
    plan = mg.Plan([(worlds[k], s, qx0, qz0, nx, nz, qy) for k, s, qx0, qz0, nx, nz, qy in reqs], tie_rule=rule)
    out = plan.split(plan.run())
    for (k, s, qx0, qz0, nx, nz, qy), got in zip(reqs, out):
        exp = oracle_grid(k[0], k[1], s, qx0, qz0, nx, nz, qy, rule)
        assert np.array_equal(got, exp), (k, s, qx0, qz0, nx, nz)


def test_batch_equals_plain_and_replays(env):
    torch = pytest.importorskip("torch")
    mg, gens, worlds = env
    reqs = mixed_requests(worlds, n=36, seed=4)
    plan = mg.Plan([(worlds[k], s, qx0, qz0, nx, nz, qy) for k, s, qx0, qz0, nx, nz, qy in reqs])
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    d_out = torch.zeros(plan.output_bytes, dtype=torch.uint8, device=dev)
    plan.run_dev(d_out.data_ptr(), stream)
    first = d_out.cpu().numpy().copy()
    for _ in range(2):  # graph replays overwrite the same bytes with the same values
        d_out.fill_(0xEE)
        plan.run_dev(d_out.data_ptr(), stream)
        assert np.array_equal(d_out.cpu().numpy(), first)
    d_out.fill_(0xEE)
    plan.run_dev(d_out.data_ptr(), stream, graph=False)
    assert np.array_equal(d_out.cpu().numpy(), first)
    # the plain form: one setup + one grid launch per request
    plain = torch.full_like(d_out, 0xEE)
    for i, (k, s, qx0, qz0, nx, nz, qy) in enumerate(reqs):
        worlds[k].quart_grid_seed_dev(s, qx0, qz0, nx, nz, qy, 0, plain.data_ptr() + plan.offset(i), stream)
    assert np.array_equal(plain.cpu().numpy(), first)
    # every tile shape the autotuner tries gives the same ids
    for shape in range(4):
        plan.shape = shape
        d_out.fill_(0xEE)
        plan.run_dev(d_out.data_ptr(), stream)
        assert np.array_equal(d_out.cpu().numpy(), first), shape
    ms = plan.autotune(d_out.data_ptr(), reps=1)
    assert ms > 0 and 0 <= plan.shape < 4
    plan.run_dev(d_out.data_ptr(), stream)
    assert np.array_equal(d_out.cpu().numpy(), first)


def test_batch_config4_sample(env):
    """A 200-request prefix of the uneven mixed batch workload (SplitMix64(3)), checked against the oracle."""
    import bench

    mg, gens, worlds = env
    reqs = bench.config4_requests(200)
    plan = mg.Plan([(worlds[(v, d)], s, qx0, qz0, n, n, qy) for v, d, s, qx0, qz0, n, qy in reqs])
    out = plan.split(plan.run())
    for i in range(0, 200, 7):
        v, d, s, qx0, qz0, n, qy = reqs[i]
        exp = O.World(ge.data_root(), v, d.split(":")[1]).quart_grid(s, qx0, qz0, n, n, qy, O.TIE_ENGINE)
        assert np.array_equal(out[i], exp), reqs[i]


def test_batch_presets_versions_extremes(env):
    """Plans over worlds the uneven batch does not draw: 26.4-snapshot-2, amplified and large_biomes, at
    coordinates near the +-30M-block world border, single cells, rows and a 700 x 3 strip; CHUNK_CELL too."""
    mg, gens, worlds = env
    wl = {("26.4-snapshot-2", "minecraft:overworld", "normal"): gens["26.4-snapshot-2"].world("minecraft:overworld", "normal", 0),
          ("26.1", "minecraft:overworld", "amplified"): gens["26.1"].world("minecraft:overworld", "amplified", 0),
          ("26.3", "minecraft:overworld", "large_biomes"): gens["26.3"].world("minecraft:overworld", "large_biomes", 0),
          ("26.2", "minecraft:the_end", "normal"): gens["26.2"].world("minecraft:the_end", "normal", 0)}
    cases = [(-7_499_990, 7_499_000, 24, 40), (7_499_000, -7_499_990, 1, 1), (-3, -2, 700, 3), (123, -456, 1, 65)]
    reqs = []
    for i, key in enumerate(wl):
        for j, (qx0, qz0, nx, nz) in enumerate(cases):
            reqs.append((key, (i * 7919 + j * 104729) * (-1) ** j, qx0, qz0, nx, nz, 16 if j % 2 else -10))
    for rule in (0, 2):
        plan = mg.Plan([(wl[k], s, qx0, qz0, nx, nz, qy) for k, s, qx0, qz0, nx, nz, qy in reqs], tie_rule=rule)
        out = plan.split(plan.run())
        for (k, s, qx0, qz0, nx, nz, qy), got in zip(reqs, out):
            ow = O.World(ge.data_root(), k[0], k[1].split(":")[1], k[2])
            if rule == 2 and not k[1].endswith("the_end"):
                exp = ow.chunk_grid(s, qx0, qz0, nx, nz, qy)
            else:
                exp = ow.quart_grid(s, qx0, qz0, nx, nz, qy, O.TIE_ENGINE)
            assert np.array_equal(got, exp), (k, s, qx0, qz0, nx, nz, rule)


def test_plan_outlives_freed_world_and_orders_runs(env):
    """A plan keeps its worlds alive past mcgen_world_free; runs of one plan on two streams with no ordering
    between them are serialised by the library (they share the plan's lattice pool and tile counter), so
    both outputs are exact; freeing the plan right after queuing runs does not block and leaves them exact."""
    torch = pytest.importorskip("torch")
    mg, gens, worlds = env
    dev = torch.device("cuda", 0)
    w = gens["26.2"].world("minecraft:overworld", "normal", 0)
    reqs = [(w, 9000 + i, -300 + 37 * i, 200 - 11 * i, 50 + 7 * i, 33, 16) for i in range(12)]
    plan = mg.Plan(reqs)
    w.close()  # the plan still uses the world's description and tree
    ow = O.World(ge.data_root(), "26.2", "overworld")
    exp = np.concatenate([ow.quart_grid(s, qx0, qz0, nx, nz, qy, O.TIE_ENGINE).ravel()
                          for _, s, qx0, qz0, nx, nz, qy in reqs])
    a, b = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    oa = torch.zeros(plan.output_bytes, dtype=torch.uint8, device=dev)
    ob = torch.zeros_like(oa)
    for _ in range(3):
        plan.run_dev(oa.data_ptr(), a.cuda_stream)
        plan.run_dev(ob.data_ptr(), b.cuda_stream, graph=False)
    plan.close()
    torch.cuda.synchronize(dev)
    assert np.array_equal(oa.cpu().numpy(), exp)
    assert np.array_equal(ob.cpu().numpy(), exp)
