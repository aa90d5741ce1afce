"""The served form: continuous batching with a device noise-state cache.

Each request's ids must be the same whether it is served alone or mixed with concurrent requests from
several threads (different versions, dimensions, sizes, repeated seeds), and equal to the oracle; a small
HBM budget must evict (LRU) without changing any result."""
import ctypes as C
import threading

import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import oracle as O

pytestmark = pytest.mark.gpu
VERSIONS = ["26.1", "26.2", "26.3"]
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


def requests(worlds, n, seed):
    rng = np.random.default_rng(seed)
    keys = sorted(worlds)
    seeds = [int(x) for x in rng.integers(-2**63, 2**63 - 1, 7)]  # few seeds: cache hits and in-flight sharing
    out = []
    for i in range(n):
        k = keys[int(rng.integers(len(keys)))]
        side = int(rng.integers(1, 90))
        out.append((k, seeds[int(rng.integers(len(seeds)))], int(rng.integers(-5000, 5000)),
                    int(rng.integers(-5000, 5000)), side, max(1, side // 2 + int(rng.integers(0, 9))), 16))
    return out


def test_alone_equals_mixed(env):
    mg, gens, worlds = env
    reqs = requests(worlds, 120, 1)
    srv = mg.Server(hbm_budget_bytes=256 << 20, max_inflight=3)
    alone = []
    for k, s, qx0, qz0, nx, nz, qy in reqs:  # one at a time
        ids, _ = srv.wait(srv.submit(worlds[k], s, qx0, qz0, nx, nz, qy))
        alone.append(ids.copy())
    mixed = [None] * len(reqs)

    def client(part):
        tickets = [(i, srv.submit(worlds[reqs[i][0]], *reqs[i][1:])) for i in part]
        for i, t in tickets:
            mixed[i] = srv.wait(t)[0]

    threads = [threading.Thread(target=client, args=(list(range(j, len(reqs), 4)),)) for j in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    st = srv.stats()
    srv.close()
    for i, (a, b) in enumerate(zip(alone, mixed)):
        assert np.array_equal(a, b), reqs[i]
    for i in range(0, len(reqs), 9):
        (v, d), s, qx0, qz0, nx, nz, qy = reqs[i]
        exp = O.World(ge.data_root(), v, d.split(":")[1]).quart_grid(s, qx0, qz0, nx, nz, qy, O.TIE_ENGINE)
        assert np.array_equal(alone[i], exp), reqs[i]
    assert st["batches"] < 2 * len(reqs)  # the mixed phase was batched
    assert st["cache_hits"] > 0


def test_small_budget_evicts(env):
    """A budget of a few Overworld slots forces LRU eviction; every result is still exact."""
    mg, gens, worlds = env
    srv = mg.Server(hbm_budget_bytes=4 * 48 * 352 * 16 // 12 + 64 * 352, max_inflight=2, max_batch=3)
    rng = np.random.default_rng(7)
    w = worlds[("26.3", "minecraft:overworld")]
    ow = O.World(ge.data_root(), "26.3", "overworld")
    tickets = []
    for i in range(24):
        s = int(rng.integers(-2**62, 2**62))
        tickets.append((s, srv.submit(w, s, -40, 30, 24, 16, 16)))
    for s, t in tickets:
        ids, lat = srv.wait(t)
        assert np.array_equal(ids, ow.quart_grid(s, -40, 30, 24, 16, 16, O.TIE_ENGINE))
        assert lat >= 0
    st = srv.stats()
    srv.close()
    assert st["cache_evictions"] > 0


def test_wait_timeout_and_ticket_rules(env):
    """A wait that runs out returns MCGEN_E_CANCEL and the ticket stays valid; a ticket is waited for once;
    unknown tickets and a missing output buffer are refused."""
    mg, gens, worlds = env
    srv = mg.Server(hbm_budget_bytes=64 << 20, max_inflight=1)
    w = worlds[("26.1", "minecraft:overworld")]
    big = srv.submit(w, 123, -256, -256, 512, 512, 16)   # long enough that a 0 ms wait usually runs out
    small = srv.submit(w, 124, 0, 0, 8, 8, 16)
    try:
        srv.wait(small, 0)
    except mg.McError as e:
        assert e.code == mg.MCGEN_E_CANCEL
    ids, lat = srv.wait(big)
    exp = O.World(ge.data_root(), "26.1", "overworld").quart_grid(123, -256, -256, 512, 512, 16, O.TIE_ENGINE)
    assert np.array_equal(ids, exp) and lat > 0
    if small in srv._keep:
        ids2, _ = srv.wait(small)
        assert np.array_equal(ids2, O.World(ge.data_root(), "26.1", "overworld").quart_grid(124, 0, 0, 8, 8, 16, O.TIE_ENGINE))
    with pytest.raises(mg.McError) as e:
        srv.wait(big)                                      # already collected
    assert e.value.code == mg.MCGEN_E_ARG
    L = mg.load()
    req = mg.McGb300Request(w.handle, 5, 0, 0, 4, 4, 16)
    t = C.c_longlong()
    assert L.mcgen_gb300_server_submit(srv._h, C.byref(req), None, C.byref(t)) == mg.MCGEN_E_ARG
    srv.close()


def test_failed_batch_leaves_no_partial_state(env):
    """A batch that fails while forming (an allocation failure injected on the host) fails its own requests
    and takes back the cache entries it had created: the same seeds asked again are rebuilt and exact, and no
    request ever comes back MCGEN_OK with wrong ids.  A failure other than an allocation stops the server:
    pending and later requests fail with it."""
    mg, gens, worlds = env
    w = worlds[("26.3", "minecraft:overworld")]
    ow = O.World(ge.data_root(), "26.3", "overworld")
    srv = mg.Server(hbm_budget_bytes=64 << 20, max_inflight=1)
    seeds = [1111, -2222, 3333, 4444]
    exp = {s: ow.quart_grid(s, -20, 12, 16, 16, 16, O.TIE_ENGINE) for s in seeds}
    srv.fail_next(mg.MCGEN_E_NOMEM)
    tickets = [(s, srv.submit(w, s, -20, 12, 16, 16, 16)) for s in seeds]
    failed = 0
    for s, t in tickets:
        try:
            ids, _ = srv.wait(t)
        except mg.McError as e:
            assert e.code == mg.MCGEN_E_NOMEM
            failed += 1
            continue
        assert np.array_equal(ids, exp[s])
    assert failed >= 1
    for s in seeds:  # hits would read lattices that were never built if the entries had stayed
        ids, _ = srv.wait(srv.submit(w, s, -20, 12, 16, 16, 16))
        assert np.array_equal(ids, exp[s])
    srv.fail_next(mg.MCGEN_E_INTERNAL)
    with pytest.raises(mg.McError) as e:
        srv.wait(srv.submit(w, seeds[0], -20, 12, 16, 16, 16))
    assert e.value.code == mg.MCGEN_E_INTERNAL
    with pytest.raises(mg.McError) as e:
        srv.submit(w, seeds[1], -20, 12, 16, 16, 16)
    assert e.value.code == mg.MCGEN_E_INTERNAL
    srv.close()


def test_world_freed_while_served(env):
    """A world freed while its requests are pending stays alive until they complete; the cache is keyed by
    the world's identity, so a new world (possibly at the same address) never hits the old one's lattices."""
    mg, gens, worlds = env
    srv = mg.Server(hbm_budget_bytes=64 << 20, max_inflight=2)
    w = gens["26.1"].world("minecraft:overworld", "normal", 0)
    t = [srv.submit(w, 77 + i, 100, -50, 40, 40, 16) for i in range(6)]
    w.close()
    ow = O.World(ge.data_root(), "26.1", "overworld")
    for i, tk in enumerate(t):
        ids, _ = srv.wait(tk)
        assert np.array_equal(ids, ow.quart_grid(77 + i, 100, -50, 40, 40, 16, O.TIE_ENGINE))
    # a world of another preset with the same seeds: its own lattices and tree, not the freed world's
    w2 = gens["26.1"].world("minecraft:overworld", "large_biomes", 0)
    lb = O.World(ge.data_root(), "26.1", "overworld", "large_biomes")
    for i in range(3):
        ids, _ = srv.wait(srv.submit(w2, 77 + i, 100, -50, 40, 40, 16))
        assert np.array_equal(ids, lb.quart_grid(77 + i, 100, -50, 40, 40, 16, O.TIE_ENGINE))
    srv.close()


def test_native_replay(env):
    """mcgen_gb300_server_replay: an open-loop schedule replayed by the library's native submitter; every
    request's ids equal the oracle's, latencies (from each scheduled arrival) are positive."""
    mg, gens, worlds = env
    rng = np.random.default_rng(17)
    n = 60
    keys = sorted(worlds)
    wi = rng.integers(0, len(keys), n)
    seeds = rng.integers(-2**62, 2**62, n)
    side = rng.integers(4, 40, n)
    qx0, qz0 = rng.integers(-3000, 3000, n), rng.integers(-3000, 3000, n)
    arrival = np.cumsum(rng.exponential(1 / 3000.0, n))
    reqs = mg.RequestArray.from_index([worlds[k] for k in keys], wi, seeds, qx0, qz0, side, side, 16)
    off = np.concatenate([[0], np.cumsum(side * side)[:-1]])
    out = np.zeros(int((side * side).sum()), np.uint8)
    srv = mg.Server(hbm_budget_bytes=64 << 20, max_inflight=2)
    lat, elapsed = srv.replay(reqs, arrival, out, off)
    srv.close()
    assert lat.shape == (n,) and (lat > 0).all() and elapsed >= arrival[-1]
    for i in range(n):
        v, d = keys[wi[i]]
        exp = O.World(ge.data_root(), v, d.split(":")[1]).quart_grid(int(seeds[i]), int(qx0[i]), int(qz0[i]),
                                                                     int(side[i]), int(side[i]), 16, O.TIE_ENGINE)
        assert np.array_equal(out[off[i]:off[i] + side[i] ** 2].reshape(side[i], side[i]), exp), i
