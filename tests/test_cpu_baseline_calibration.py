"""Calibration of the CPU baseline: the oracle port (what bench.py times on the GPU host, which has no
reference source tree) against the reference engine's own CPU path, mcg_ref_points
(engine/cuda/mcg_host.c:86-133), built from the reference sources where they are mounted (oracle/build.py).

Same inputs (the many-seeds x 8-points shape: SplitMix64(1) seeds, SplitMix64(101) points), same thread
count, identical outputs; the printed time ratio (port / reference) says how far the port's timing can be
from the reference's own (run with -s to see it).  Skipped where the reference tree is absent."""
import ctypes as C
import os
import time

import numpy as np
import pytest

import bench
from oracle import build as ob
from oracle import oracle as O


def _best(f, reps=3):
    t = 1e30
    for _ in range(reps):
        t0 = time.perf_counter()
        f()
        t = min(t, time.perf_counter() - t0)
    return t


@pytest.mark.parametrize("version,vi", [("26.3", 2), ("26.1", 0)])
def test_port_time_against_reference_engine(data_root, version, vi):
    path = ob.build_reference()
    if path is None:
        pytest.skip("reference source tree not mounted")
    threads = min(8, os.cpu_count() or 1)
    C.CDLL("libgomp.so.1").omp_set_num_threads(threads)  # the reference's parallel loop over seeds
    os.environ["MCGEN_ROOT"] = ob.REFERENCE_ROOT
    L = C.CDLL(path)
    L.ref_open.restype = C.c_void_p
    L.ref_open.argtypes = [C.c_int, C.c_int, C.c_char_p]
    L.ref_close.argtypes = [C.c_void_p]
    L.ref_points.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    h = L.ref_open(vi, 0, b"normal")
    assert h
    seeds, pts = bench.config2_inputs(8192)
    ref_b = np.zeros((seeds.size, len(pts)), np.uint8)
    ref_t = np.zeros((seeds.size, len(pts), 6), np.int32)
    t_ref = _best(lambda: L.ref_points(h, seeds.ctypes.data, seeds.size, pts.ctypes.data, len(pts), ref_b.ctypes.data,
                                       ref_t.ctypes.data))
    L.ref_close(h)
    w = O.World(data_root, version, "overworld")
    out = {}

    def port():
        out["r"] = w.points(seeds, pts, threads=threads, want_targets=True)

    t_port = _best(port)
    b, tg = out["r"]
    assert np.array_equal(b, ref_b)
    assert np.array_equal(tg, ref_t)
    ratio = t_port / t_ref
    print(f"\n{version}: {seeds.size} seeds x {len(pts)} points, {threads} threads: reference {t_ref * 1e3:.1f} ms, "
          f"port {t_port * 1e3:.1f} ms, port / reference = {ratio:.2f}")
    assert 0.33 < ratio < 3.0
