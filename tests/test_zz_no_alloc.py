"""The allocation-free seeds x points entry point (mcgen_gb300_seed_points_noalloc).

It exists for callers that cannot let the library allocate device memory (an application-owned arena, a
latency-critical loop, no allocation after set-up): the per-seed lattices go to a fixed 16 MiB array in
the library instead of per-call scratch.  Its output must equal the ordinary entry point's bit for bit,
call after call (the array keeps the previous call's contents), and it must refuse seed counts that do not
fit.  This file is collected last so that, if it fails, a run stopping at the first failure has already run
every other test.
"""
import ctypes as C

import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _call(mg, w, d_seeds, ns, d_pts, np_, d_out, d_tg, stream):
    return mg.load().mcgen_gb300_seed_points_noalloc(w.handle, d_seeds, ns, d_pts, np_, d_out, d_tg, stream)


# 16 MiB // (lattices per seed x 352-byte lattice): 46 Overworld, 8 Nether, 1 End lattice per seed
@pytest.mark.parametrize("dim,max_seeds", [("minecraft:overworld", 1036), ("minecraft:the_nether", 5957),
                                           ("minecraft:the_end", 47662)])
def test_noalloc_matches_allocating_entry(dim, max_seeds):
    torch = pytest.importorskip("torch")
    mg = ge.package()
    mg.load()
    if mg.device_count() < 1:
        pytest.fail("no CUDA device")
    gen = mg.Generator.open(ge.data_root(), "26.3")
    w = gen.world(dim, "normal", 0)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(2024)
    pts = np.stack([rng.integers(-20000, 20000, 8), rng.integers(-16, 80, 8), rng.integers(-20000, 20000, 8)],
                   1).astype(np.int32)
    d_pts = torch.from_numpy(pts).to(dev)
    # two calls in a row with different seeds (and sizes): each must match the allocating entry point,
    # so nothing stale from the previous call may leak into the next
    for ns in (max_seeds, 257):
        seeds = rng.integers(-2**63, 2**63 - 1, size=ns, dtype=np.int64)
        exp, exp_tg = w.seed_points(seeds, pts, want_targets=True)  # also puts the world on the device
        d_seeds = torch.from_numpy(seeds).to(dev)
        d_out = torch.full((ns * len(pts),), 0xEE, dtype=torch.uint8, device=dev)
        d_tg = torch.full((ns * len(pts) * 6,), -7, dtype=torch.int32, device=dev)
        rc = _call(mg, w, d_seeds.data_ptr(), ns, d_pts.data_ptr(), len(pts), d_out.data_ptr(), d_tg.data_ptr(),
                   stream.cuda_stream)
        assert rc == mg.MCGEN_OK
        torch.cuda.synchronize(dev)
        got = d_out.cpu().numpy().reshape(ns, len(pts))
        got_tg = d_tg.cpu().numpy().reshape(ns, len(pts), 6)
        assert np.array_equal(got, exp)
        assert np.array_equal(got_tg, exp_tg)
        # and the oracle on a stride sample of the seeds (about 64 of them)
        pick = np.arange(0, ns, max(1, ns // 64))
        ora, ora_tg = O.World(ge.data_root(), "26.3", dim.split(":")[1]).points(seeds[pick], pts, want_targets=True)
        assert np.array_equal(got[pick], ora)
        assert np.array_equal(got_tg[pick], ora_tg)
    # one seed more than the fixed scratch holds is refused, and nothing is written
    big = torch.zeros(max_seeds + 1, dtype=torch.int64, device=dev)
    d_out = torch.full(((max_seeds + 1) * len(pts),), 0xEE, dtype=torch.uint8, device=dev)
    rc = _call(mg, w, big.data_ptr(), max_seeds + 1, d_pts.data_ptr(), len(pts), d_out.data_ptr(), None,
               stream.cuda_stream)
    assert rc == mg.MCGEN_E_ARG
    torch.cuda.synchronize(dev)
    assert int((d_out != 0xEE).sum()) == 0


def test_noalloc_argument_checks():
    mg = ge.package()
    mg.load()
    L = mg.load()
    assert L.mcgen_gb300_seed_points_noalloc(None, None, 1, None, 1, None, None, None) == mg.MCGEN_E_ARG
    gen = mg.Generator.open(ge.data_root(), "26.1")
    w = gen.world("minecraft:overworld", "normal", 5)  # never used on the device: refused, not allocated
    dummy = C.c_void_p(16)
    assert L.mcgen_gb300_seed_points_noalloc(w.handle, dummy, 1, dummy, 1, dummy, None, None) == mg.MCGEN_E_ARG
