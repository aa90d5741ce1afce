#!/usr/bin/env python3
"""Benchmark of the bit-exact biome path on GB300 (one JSON line on rank 0).

Workloads (synthetic inputs with the shapes of the published configurations):
  seeds8   Overworld 26.3, 65,536 SplitMix64(1) world seeds x the same 8 points
           (x, z uniform in [-10000, 10000] blocks, y uniform in [-64, 320]; quart cells = block >> 2):
           per-seed noise setup + climate + R-tree, ENGINE tie rule.  [65536, 8] biome ids.
  grid256  Overworld 26.3, seed 12345, mcgen_biome_grid 256 x 256 cells, x,z in [-512, 512) step 4,
           y = 64 (BiomeManager zoom + chunk-cell ties).  65,536 samples per step.
  dims4096 Nether 26.3 and End 26.3: 4,096 SplitMix64(2) seeds x a 64 x 64 quart grid at y = 64 each, one
           batched launch per dimension.
  batch10k (default) the uneven mixed batch: 10,000 SplitMix64(3) requests (versions 26.1/26.2/26.3,
           Overworld:Nether:End 6:2:2, side log-uniform in [16, 512) quart cells), one persistent launch, against
           the plain form (one setup + one grid launch per request).  e2e: per step a plan is built from the
           host request list, run into pinned host memory and freed.  The default line also carries `configs`:
           C1 (grid256 and its quart form), C2 (seeds8), C3 (dims4096) and C5 (serve at 2,000 requests/s for
           60 s), each with value, e2e, cpu_baseline and parity (--no-configs: the headline only).
  serve    open-loop Poisson streams at --rates requests/s for --duration s each (SplitMix64(4), Zipf(1.1) over
           50,000 seeds) against the continuous-batching server; p50/p99 latency from each request's scheduled
           arrival, cache hit rate, mean batch.

Parity: the CPU-baseline leg runs the oracle (the reference algorithm restated) on a sample of the same
workload; its outputs are also compared with the GPU's timed outputs (`parity`: compared samples and
mismatches; every code-path class of the uneven batch).

A step is one pass of the workload.  `value` times steps with inputs resident in HBM through the
device-pointer entry points; `e2e` times the same work through the host-buffer C ABI calls
(mcgen_gb300_seed_points / mcgen_biome_grid) with pinned host buffers, copies included.
--impl reference times the reference algorithm on the host's cores (the CPU oracle, which is the
reference engine's CPU path restated; the reference's own build needs its source tree, which this host
does not have) on a bounded sample of the same workload.

Multi-GPU: replicas only (the path has no exchange step); each rank runs the full workload and
`value` = all ranks' samples / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

METRIC = "bit-exact biome samples/sec"
UNIT = "samples/s"
GOLDEN = 0x9E3779B97F4A7C15


def splitmix64(state: int, n: int) -> np.ndarray:
    """n outputs of SplitMix64 from `state` (z += golden; Stafford-13 mix), as uint64."""
    with np.errstate(over="ignore"):
        z = (np.uint64(state) + np.arange(1, n + 1, dtype=np.uint64) * np.uint64(GOLDEN)).astype(np.uint64)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def config2_inputs(n_seeds: int = 65536):
    """65,536 SplitMix64(1) seeds and 8 points from SplitMix64(101): x,z = -10000 + r % 20001,
    y = -64 + r % 385 (blocks), quart cell = block >> 2."""
    seeds = splitmix64(1, n_seeds).view(np.int64)
    r = splitmix64(101, 24).astype(np.uint64)
    x = -10000 + (r[0:8] % np.uint64(20001)).astype(np.int64)
    y = -64 + (r[8:16] % np.uint64(385)).astype(np.int64)
    z = -10000 + (r[16:24] % np.uint64(20001)).astype(np.int64)
    pts = np.stack([x >> 2, y >> 2, z >> 2], 1).astype(np.int32)
    return seeds, pts


def config3_inputs(n_seeds: int = 4096):
    """Other dimensions: 4,096 SplitMix64(2) seeds, each with a 64 x 64 quart grid at y=64 whose corner is drawn
    from SplitMix64(102) uniformly in [-30000, 30000) blocks (quart = block >> 2), so that the End grids sample
    the outer islands and not only the central island (|chunk| <= 64)."""
    seeds = splitmix64(2, n_seeds).view(np.int64)
    r = splitmix64(102, 2 * n_seeds).reshape(n_seeds, 2)
    origins = ((-30000 + (r % np.uint64(60000)).astype(np.int64)) >> 2).astype(np.int32)
    return seeds, origins


C4_VERSIONS = ("26.1", "26.2", "26.3")
C4_DIMS = ("minecraft:overworld",) * 6 + ("minecraft:the_nether",) * 2 + ("minecraft:the_end",) * 2


def config4_requests(n: int = 10000, state: int = 3):
    """The uneven mixed batch: n requests from SplitMix64(state), six draws each -- seed; version uniform over
    26.1/26.2/26.3; dimension Overworld:Nether:End = 6:2:2; square side floor(16 * 32^u) quart cells (u uniform
    in [0,1): log-uniform in [16, 512)); origin x, z uniform in [-30000, 30000] blocks (quart = block >> 2);
    y = 64 (quart 16).  Returns (version, dimension, seed, qx0, qz0, side, qy) tuples."""
    r = splitmix64(state, 6 * n).reshape(n, 6)
    out = []
    for i in range(n):
        seed = int(r[i, 0].astype(np.int64))
        version = C4_VERSIONS[int(r[i, 1] % np.uint64(3))]
        dim = C4_DIMS[int(r[i, 2] % np.uint64(10))]
        u = float(r[i, 3] >> np.uint64(11)) * 2.0 ** -53
        side = int(16.0 * 32.0 ** u)
        x = -30000 + int(r[i, 4] % np.uint64(60001))
        z = -30000 + int(r[i, 5] % np.uint64(60001))
        out.append((version, dim, seed, x >> 2, z >> 2, side, 16))
    return out


# ------------------------------------------------------------------------------------------ helpers
def max_over_ranks(x: float, world: int, device) -> float:
    """The slowest rank's time: replicas run independently and the job takes as long as its slowest."""
    if world <= 1:
        return float(x)
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class ClockSampler:
    """nvidia-smi SM clock / throttle samples every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.t:
                self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [s.strip() for s in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = max(mx, float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def gpu_peaks(mg) -> dict:
    """Measured pipe rates (Gop/s) on this device; the host file gives only HBM and bf16 GEMM."""
    return {k: round(mg.pipe_rate(k), 1) for k in ("fp32_fma", "fp64_fma", "fp64_add", "int32_mad",
                                                   "cvt_f64_floor_s32", "cvt_s32_f64", "cvt_f64_f32", "int64_mad",
                                                   "cvt_s64_f64", "cvt_f32_f64")}


# Lattice (octave) samples per biome sample: 52 in the Overworld (six NormalNoises, two stacks each, with
# the shift noise sampled twice), 8 in the Nether; the oracle's work counter pins both numbers.
OCTAVES_PER_SAMPLE = {"minecraft:overworld": 52, "minecraft:the_nether": 8, "minecraft:the_end": 0}
# FP64 operations per sample as the kernels compute them.  Float branch (26.3+): the two rounded coordinate
# adds of every octave sample (Overworld 52 x 2, Nether 8 x 2).  Double branch (26.1/26.2), Overworld: the
# shift noise's 12 octave samples exactly in double, their splits and smoothsteps taken from the tile's
# table (29 each: 8 conversions of the exact gradient sums and differences, 4 first-level lerp products and
# sums, 3 lerps of 3, the product undoing the 2^52 scale, the amplitude products and sum), the table itself
# (6 lattices x 48 entries of 8 per 128-cell tile: 18 per sample), and the 40 climate octave samples in
# 59-bit fixed point with only their 2 coordinate adds on the FP64 pipe (the screens and ridges_folded run
# on the integer and conversion pipes): 348 + 18 + 80 = 446.  Nether: 8 x 2 = 16.  The rare values the
# screen leaves to the exact double path and the End's simplex are left out, so the model is a lower bound.
FP64_PER_SAMPLE = {("double", "minecraft:overworld"): 446, ("double", "minecraft:the_nether"): 16,
                   ("float", "minecraft:overworld"): 104, ("float", "minecraft:the_nether"): 16,
                   ("double", "minecraft:the_end"): 0, ("float", "minecraft:the_end"): 0}
DOUBLE_BRANCH = ("26.1", "26.2")


def batch_fp64_ops(reqs) -> float:
    return float(sum(n * n * FP64_PER_SAMPLE[("double" if v in DOUBLE_BRANCH else "float", d)]
                     for v, d, s, qx0, qz0, n, qy in reqs))


# Algorithmic work per launch of each kernel, counted from the reference algorithm:
# (work units per launch, unit name, pipe peak key).
# DRAM bytes (read + write) per work unit of a launch, from one ncu capture each: k_batch per sample
# (the first 4,000 requests of the uneven batch), k_ow_seed_climate per seed (4,096 seeds x 8 points).
DRAM_BYTES_PER_UNIT = {"k_batch": (72375552 + 1504797696) / 147087943, "k_ow_seed_climate": 83200 / 4096}
K_BATCH_TRAFFIC_NOTE = ("DRAM bytes read + written per sample in an ncu capture of one k_batch<8, 8> launch over the "
                        "first 4,000 requests (147 M samples, an output larger than L2) x this launch's samples; "
                        "the writes are mostly local-memory write-back (register spills), the ids 1 B per sample")
# pipe utilisation of k_batch<8, 8> from ncu (sm__inst_executed_pipe_*, issue active) on a 300-request launch
K_BATCH_PIPES = {"fp64": 0.547, "integer_alu": 0.546, "issue_active": 0.682}


def kernel_work(kernel: str, seeds8: bool, ns: int, np_: int, ntables: int) -> tuple[float, str, str] | None:
    # Integer ALU work of the per-seed setup, which bounds both kernels below (the fused kernel's ALU pipe
    # is its busiest): per lattice 256 Fisher-Yates steps, each one Xoroshiro128++ draw (16 32-bit ALU ops:
    # two 64-bit adds, three 64-bit rotates, a shift and two 3-input xors), the Lemire bound (3) and the
    # swap addressing (2); plus three nextDouble draws (16 + 4 each).
    per_lattice = 256 * (16 + 3 + 2) + 3 * 20
    if kernel in ("k_setup_xo", "k_ow_seed_climate"):
        return float(ns * ntables * per_lattice), "Gop/s", "int32_mad"
    return None


def run_gb300(args, rank, world, local_rank):
    import torch

    import __graft_entry__ as ge

    mg = ge.package()
    mg.load()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    gen = mg.Generator.open(ge.data_root(), "26.3")
    if args.workload == "seeds8":
        seeds, pts = config2_inputs(args.seeds)
        w = gen.world("minecraft:overworld", "normal", 0)
        samples = seeds.size * len(pts)
        d_seeds = torch.from_numpy(seeds).to(dev)
        d_pts = torch.from_numpy(pts).to(dev)
        d_out = torch.empty(samples, dtype=torch.uint8, device=dev)
        h_seeds = torch.from_numpy(seeds).pin_memory()
        h_pts = torch.from_numpy(pts).pin_memory()
        h_out = torch.empty(samples, dtype=torch.uint8).pin_memory()
        nt = 46

        def dev_step(stream):
            w.seed_points_dev(d_seeds.data_ptr(), seeds.size, d_pts.data_ptr(), len(pts), d_out.data_ptr(), 0, stream)

        def host_step():
            L = mg.load()
            rc = L.mcgen_gb300_seed_points(w.handle, h_seeds.data_ptr(), seeds.size, h_pts.data_ptr(), len(pts),
                                           h_out.data_ptr(), None)
            if rc:
                raise mg.McError(rc, "seed_points failed")

        h2d = seeds.nbytes + pts.nbytes
        d2h = samples
        config = {"workload": "Overworld 26.3 normal, 65536 SplitMix64(1) seeds x 8 fixed points "
                              "(x,z in [-10000,10000], y in [-64,320]), ENGINE tie rule",
                  "seeds": int(seeds.size), "points_per_seed": int(len(pts)), "version": "26.3",
                  "dimension": "overworld", "l2": "working set > L2 (65536 x 46 lattices = 965 MB per step)"}
    elif args.workload == "batch10k":
        return run_batch(args, rank, world, local_rank, mg, ge)
    elif args.workload == "serve":
        return run_serve(args, rank, world, local_rank, mg, ge)
    elif args.workload == "dims4096":
        return run_dims(args, rank, world, local_rank, mg, ge)
    elif args.workload == "search":
        return run_search(args, rank, world, local_rank, mg, ge)
    elif args.workload == "map2048":
        return run_map(args, rank, world, local_rank, mg, ge)
    else:
        w = gen.world("minecraft:overworld", "normal", 12345)
        nx = nz = 256
        samples = nx * nz
        d_out = torch.empty(samples, dtype=torch.uint8, device=dev)
        h_out = torch.empty(samples, dtype=torch.uint8).pin_memory()
        nt = 46
        seeds = np.array([12345])
        pts = np.zeros((1, 3))

        def dev_step(stream):
            w.biome_grid_dev(-512, -512, nx, nz, 4, 64, d_out.data_ptr(), stream)

        def host_step():
            rc = mg.load().mcgen_biome_grid(w.handle, -512, -512, nx, nz, 4, 64, h_out.data_ptr())
            if rc:
                raise mg.McError(rc, "biome_grid failed")

        h2d, d2h = 0, samples
        config = {"workload": "Overworld 26.3 normal, seed 12345, mcgen_biome_grid 256x256 x,z in [-512,512) "
                              "step 4, y=64 (zoom + chunk-cell ties)", "version": "26.3", "dimension": "overworld",
                  "l2": "L2 flushed between steps (256 MB write)"}

    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev) if args.workload == "grid256" else None

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        dev_step(sh)
    torch.cuda.synchronize(dev)
    launches0 = mg.launch_count()
    mg.profile(True)
    barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local_rank) as clk:
        if flush is None:
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            for _ in range(args.steps):
                dev_step(sh)
            ev1.record(stream)
            torch.cuda.synchronize(dev)
            ms = ev0.elapsed_time(ev1)
        else:
            ms = 0.0
            for _ in range(args.steps):
                flush.fill_(1)
                ev0 = torch.cuda.Event(enable_timing=True)
                ev1 = torch.cuda.Event(enable_timing=True)
                ev0.record(stream)
                dev_step(sh)
                ev1.record(stream)
                torch.cuda.synchronize(dev)
                ms += ev0.elapsed_time(ev1)
    barrier()
    mg.profile(False)
    prof = mg.profile_read()
    launches = mg.launch_count() - launches0
    ms_max = max_over_ranks(ms, world, dev)
    value = samples * args.steps * world / (ms_max * 1e-3)

    # end to end through the host-buffer C ABI (pinned host memory, copies inside the timed region)
    if not args.skip_extras:
        for _ in range(max(1, args.warmup)):
            host_step()
    barrier()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(0 if args.skip_extras else args.steps):
        host_step()
    torch.cuda.synchronize(dev)
    e2e_s = max(time.perf_counter() - t0, 1e-9)
    e2e = samples * args.steps * world / max_over_ranks(e2e_s, world, dev)

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32+f64+int64", "data": "synthetic (SplitMix64 seeds and points)",
           "config": dict(config, parallelism=f"replicas x{world}" if world > 1 else "single GPU"),
           "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
           "gpu_launches": int(launches)}
    if rank == 0:
        kern = {k: {"ms_total": round(v[0], 4), "launches": v[1], "avg_ms": round(v[0] / v[1], 5)} for k, v in prof.items()}
        out["kernels"] = kern
        clocks = clk.summary()
        if clocks:
            out["clocks"] = clocks
        peaks = gpu_peaks(mg) if not args.skip_extras else {}
        out["pipe_peaks_gops"] = peaks
        if prof:
            top = max(prof, key=lambda k: prof[k][0])
            wk = kernel_work(top, args.workload == "seeds8", int(seeds.size), int(len(pts)), nt)
            avg_s = prof[top][0] / prof[top][1] * 1e-3
            if wk and peaks:
                ops, unit, peak_key = wk
                achieved = ops / avg_s / 1e9
                per = DRAM_BYTES_PER_UNIT.get(top)
                out["roofline"] = {"kernel": top, "bound": peak_key, "achieved": round(achieved, 1),
                                   "peak": peaks[peak_key], "unit": unit, "frac": round(achieved / peaks[peak_key], 4),
                                   "traffic": round(per * seeds.size) if per is not None else None,
                                   "peak_source": "measured in-run (pipe microbenchmark)"}
            else:
                out["roofline"] = {"kernel": top, "bound": None, "achieved": None, "peak": None, "unit": None,
                                   "frac": None, "traffic": None}
        if not args.skip_extras:
            dev_step(sh)
            torch.cuda.synchronize(dev)
            out["cpu_baseline"], out["parity"] = cpu_baseline(args.workload, args.cpu_sample_s, d_out.cpu().numpy())
            if args.workload == "grid256":
                out["parity_quart_form"] = quart_form_parity(mg, gen, dev)
                out["quart_form"] = quart_form_rate(mg, gen, dev, args.steps, max(3, args.warmup))
    return out


def run_batch(args, rank, world, local_rank, mg, ge):
    """Uneven mixed batch: 10,000 requests in one persistent launch (plan + CUDA graph), against the plain
    form (one setup + one grid launch per request) on the same requests."""
    import torch

    dev = torch.device("cuda", local_rank)
    reqs = config4_requests(args.requests)
    if args.batch_class:  # profiling one code path: only that class's requests
        reqs = [r for r in reqs if class_of(r[0], r[1]) == args.batch_class]
    gens = {v: mg.Generator.open(ge.data_root(), v) for v in C4_VERSIONS}
    worlds = {(v, d): gens[v].world(d, "normal", 0) for v in C4_VERSIONS for d in set(C4_DIMS)}
    plan = mg.Plan([(worlds[(v, d)], s, qx0, qz0, n, n, qy) for v, d, s, qx0, qz0, n, qy in reqs])
    samples = plan.output_bytes
    d_out = torch.empty(samples, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    tuned_ms = plan.autotune(d_out.data_ptr(), reps=1)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        plan.run_dev(d_out.data_ptr(), sh)
    torch.cuda.synchronize(dev)
    launches0 = mg.launch_count()
    barrier()
    with ClockSampler(local_rank) as clk:
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            plan.run_dev(d_out.data_ptr(), sh)
        ev1.record(stream)
        torch.cuda.synchronize(dev)
        ms = ev0.elapsed_time(ev1)
    barrier()
    graph_launches = mg.launch_count() - launches0  # graph replays are not counted by the library
    ms_max = max_over_ranks(ms, world, dev)
    value = samples * args.steps * world / (ms_max * 1e-3)
    # per-kernel times: one run without the graph, under the library's event profiler
    mg.profile(True)
    plan.run_dev(d_out.data_ptr(), sh, graph=False)
    torch.cuda.synchronize(dev)
    mg.profile(False)
    prof = mg.profile_read()
    # plain form on the same requests
    plain = torch.empty_like(d_out)
    offs = [plan.offset(i) for i in range(len(reqs))]

    def plain_step():
        for i, (v, d, s, qx0, qz0, n, qy) in enumerate(reqs):
            worlds[(v, d)].quart_grid_seed_dev(s, qx0, qz0, n, n, qy, 0, plain.data_ptr() + offs[i], sh)

    plain_step()
    torch.cuda.synchronize(dev)
    pe0, pe1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    pe0.record(stream)
    plain_step()
    pe1.record(stream)
    torch.cuda.synchronize(dev)
    plain_wall = time.perf_counter() - t0
    plain_ms = max(pe0.elapsed_time(pe1), plain_wall * 1e3)
    same = bool(torch.equal(plain, d_out))
    # the reference's per-request call pattern (libmcgen/gpu/mcgpu_biome.cu:203-249: each call runs its
    # launches, synchronises and copies its ids to the host): the same launches, then a device->host copy
    # of the request's ids into pinned memory and a synchronisation, request by request
    h_plain = torch.empty(samples, dtype=torch.uint8).pin_memory()

    def plain_sync_step():
        for i, (v, d, s, qx0, qz0, n, qy) in enumerate(reqs):
            worlds[(v, d)].quart_grid_seed_dev(s, qx0, qz0, n, n, qy, 0, plain.data_ptr() + offs[i], sh)
            h_plain[offs[i]:offs[i] + n * n].copy_(plain[offs[i]:offs[i] + n * n], non_blocking=True)
            stream.synchronize()

    t0 = time.perf_counter()
    plain_sync_step()
    plain_sync_ms = (time.perf_counter() - t0) * 1e3
    # end to end through the public API, every step: the request list goes in from the host (plan_new copies
    # worlds, requests and setup lists to the device), the plan runs, the ids come back into pinned memory
    h_out = torch.empty(samples, dtype=torch.uint8).pin_memory()
    hv = h_out.numpy()
    shape = plan.shape
    # the request list as a caller keeps it for the library: one packed record array (McGb300Request[])
    wkeys = sorted(worlds)
    plan_args = mg.RequestArray.from_index([worlds[k] for k in wkeys], [wkeys.index((v, d)) for v, d, *_ in reqs],
                                           [r[2] for r in reqs], [r[3] for r in reqs], [r[4] for r in reqs],
                                           [r[5] for r in reqs], [r[5] for r in reqs], [r[6] for r in reqs])

    def e2e_step():
        p = mg.Plan(plan_args)
        p.shape = shape
        p.run(hv)
        b = p.h2d_bytes
        p.close()
        return b

    e2e_steps = 0 if args.skip_extras else min(args.steps, 5)
    h2d = e2e_step() if e2e_steps else 0
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        h2d = e2e_step()
    e2e_s = time.perf_counter() - t0
    e2e = samples * e2e_steps * world / e2e_s if e2e_steps else None
    per_step_launches = sum(v[1] for v in prof.values())
    batched_ms = ms_max / args.steps
    # batched vs plain, both device-resident (async) and both host to host (the headline: the batched e2e
    # call against the reference's per-request pattern)
    ratios = {"batched_over_plain_async": plain_ms / batched_ms}
    if e2e is not None:
        ratios["batched_over_plain"] = e2e / (samples / (plain_sync_ms * 1e-3))
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32+f64+int64", "data": "synthetic (SplitMix64(3) requests)",
           "config": {"workload": f"uneven mixed batch: {len(reqs)} SplitMix64(3) requests, versions 26.1/26.2/26.3, "
                                  "Overworld:Nether:End 6:2:2, square side log-uniform in [16,512) quart cells, origin "
                                  "uniform in [-30000,30000] blocks, y=64, ENGINE tie rule",
                      "form": "one persistent launch (CUDA graph) vs one plain launch pair per request",
                      **({"class_only": args.batch_class} if args.batch_class else {}),
                      "requests": len(reqs), "samples_per_step": samples, "tile_shape": plan.shape,
                      "autotune_ms": round(tuned_ms, 3), "l2": f"output {samples/1e6:.0f} MB per step > L2",
                      "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
           "plain": {"value": samples * world / (plain_sync_ms * 1e-3), "ms_per_step": plain_sync_ms,
                     "launches_per_step": 2 * len(reqs),
                     "form": "per request: setup + grid launch, ids copied to pinned host memory, synchronise "
                             "(the reference's per-request call pattern)"},
           "plain_async": {"value": samples * world / (plain_ms * 1e-3), "ms_per_step": plain_ms,
                           "identical_output": same,
                           "form": "per request: setup + grid launch into device memory, no synchronisation"},
           **ratios,
           "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(samples),
                   "steps": e2e_steps, "call": "mcgen_gb300_plan_new(request records) + plan_run(host buffer) + "
                                               "plan_free per step"},
           "gpu_launches": int(graph_launches) + args.steps * per_step_launches}
    if rank == 0:
        out["kernels"] = {k: {"ms_total": round(v[0], 4), "launches": v[1], "avg_ms": round(v[0] / v[1], 5)}
                          for k, v in prof.items()}
        clocks = clk.summary()
        if clocks:
            out["clocks"] = clocks
        peaks = gpu_peaks(mg) if not args.skip_extras else {}
        out["pipe_peaks_gops"] = peaks
        if "k_batch" in prof and peaks:
            ops = batch_fp64_ops(reqs)
            avg_s = prof["k_batch"][0] / prof["k_batch"][1] * 1e-3
            achieved = ops / avg_s / 1e9
            out["roofline"] = {"kernel": "k_batch", "bound": "fp64", "achieved": round(achieved, 1),
                               "peak": peaks["fp64_add"], "unit": "Gop/s", "frac": round(achieved / peaks["fp64_add"], 4),
                               "traffic": round(DRAM_BYTES_PER_UNIT["k_batch"] * samples),
                               "traffic_note": K_BATCH_TRAFFIC_NOTE,
                               "work": f"{ops:.4g} FP64 ops per launch (per-sample model of the screened evaluation)",
                               "peak_source": "measured in-run (FP64 add pipe microbenchmark)",
                               "binding_pipes": K_BATCH_PIPES}
        if args.split_classes:
            out["classes"] = batch_classes(reqs, worlds, mg, dev, stream)
        if not args.skip_extras:
            got = d_out.cpu().numpy()
            out["cpu_baseline"], out["parity"] = cpu_baseline_batch(reqs, offs, got, args.cpu_sample_s)
    return out


# code-path classes of the uneven batch (--split-classes): the double branch (26.1/26.2) and the float
# branch (26.3) of the Overworld and the Nether, and the End
BATCH_CLASSES = {
    "overworld_double": lambda v, d: d.endswith("overworld") and v in DOUBLE_BRANCH,
    "overworld_float": lambda v, d: d.endswith("overworld") and v not in DOUBLE_BRANCH,
    "nether_double": lambda v, d: d.endswith("nether") and v in DOUBLE_BRANCH,
    "nether_float": lambda v, d: d.endswith("nether") and v not in DOUBLE_BRANCH,
    "end": lambda v, d: d.endswith("end"),
}


def batch_classes(reqs, worlds, mg, dev, stream) -> dict:
    """Each class's requests as a plan of their own (autotuned), mean of 3 graph runs: where a step's time
    goes; and each class at every tile shape (register budget: 0 = 56 registers / 9 CTAs per SM, 1 = 72 / 7,
    2 = 80 / 6, 3 = 64 / 8), the table behind one shape for the whole batch."""
    import torch

    out = {}
    for name, f in BATCH_CLASSES.items():
        sub = [r for r in reqs if f(r[0], r[1])]
        if not sub:
            continue
        plan = mg.Plan([(worlds[(v, d)], s, qx0, qz0, n, n, qy) for v, d, s, qx0, qz0, n, qy in sub])
        d_out = torch.empty(plan.output_bytes, dtype=torch.uint8, device=dev)
        plan.autotune(d_out.data_ptr(), reps=1)
        tuned = plan.shape

        def timed(shape):
            plan.shape = shape
            plan.run_dev(d_out.data_ptr(), stream.cuda_stream)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(3):
                plan.run_dev(d_out.data_ptr(), stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            return e0.elapsed_time(e1) / 3

        per_shape = {str(k): round(timed(k), 3) for k in range(4)}  # every register budget, for the table
        ms = timed(tuned)
        out[name] = {"requests": len(sub), "samples": plan.output_bytes, "ms": round(ms, 3),
                     "ns_per_sample": round(ms * 1e6 / plan.output_bytes, 4), "tile_shape": tuned,
                     "ms_per_shape": per_shape}
        plan.close()
    return out


def class_of(v: str, d: str) -> str:
    for name, f in BATCH_CLASSES.items():
        if f(v, d):
            return name
    raise ValueError((v, d))


def cpu_baseline_batch(reqs, offs, got, budget_s: float, stride: int = 10) -> tuple[dict, dict]:
    """The reference algorithm (oracle port) on the host's cores over a stride sample of the requests (every
    `stride`-th request of each code-path class, until the class's share of the time budget is used), and
    the same outputs as the parity check of the GPU's timed output `got` (requests at offsets `offs`).
    The rate is weighted by the whole batch's samples per class: total samples / sum over classes of the
    class's samples / its CPU rate, so a sample's class mix does not bias it.  Returns (cpu_baseline, parity)."""
    import __graft_entry__ as ge
    from oracle import oracle as O

    cores = os.cpu_count() or 1
    worlds = {}
    total = {}
    for v, d, s, qx0, qz0, n, qy in reqs:
        c = class_of(v, d)
        total[c] = total.get(c, 0) + n * n
    all_samples = sum(total.values())
    rate, detail = {}, {}
    compared = mismatches = nreq = 0
    bad = []
    for c in BATCH_CLASSES:
        idx = [i for i, r in enumerate(reqs) if class_of(r[0], r[1]) == c][::stride]
        if not idx:
            continue
        share = budget_s * total[c] / all_samples
        t_cls, cells, done = 0.0, 0, 0
        for i in idx:
            v, d, s, qx0, qz0, n, qy = reqs[i]
            if (v, d) not in worlds:
                worlds[(v, d)] = O.World(ge.data_root(), v, d.split(":")[1])
            t0 = time.perf_counter()
            exp = worlds[(v, d)].quart_grid(s, qx0, qz0, n, n, qy, O.TIE_ENGINE, threads=cores)
            t_cls += time.perf_counter() - t0
            m = int(np.count_nonzero(got[offs[i]:offs[i] + n * n] != exp.ravel()))
            mismatches += m
            if m and len(bad) < 8:
                bad.append(i)
            compared += n * n
            cells += n * n
            done += 1
            if t_cls > share and done >= 4:
                break
        rate[c] = cells / t_cls
        nreq += done
        detail[c] = {"requests": done, "samples": cells, "s": round(t_cls, 2), "samples_per_s": round(rate[c])}
    value = all_samples / sum(total[c] / rate[c] for c in total)
    base = {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"every {stride}th request of each code-path class until its share of a {budget_s:.0f} s "
                      f"budget ({nreq} requests, {compared} samples), rows over threads; rate weighted by the full "
                      "batch's samples per class", "classes": detail}
    parity = {"against": "oracle (the reference engine's CPU algorithm restated, pinned to the reference's golden "
                         "vectors)", "requests": nreq, "compared_samples": compared, "mismatches": mismatches,
              "classes": sorted(detail), "sample": f"every {stride}th request per class (the CPU baseline's outputs) "
                                                  "against the timed run's output", "first_bad_requests": bad}
    return base, parity


def zipf_table(n: int = 50000, s: float = 1.1) -> np.ndarray:
    w = np.arange(1, n + 1, dtype=np.float64) ** -s
    return np.cumsum(w) / w.sum()


def config5_stream(rate: float, duration: float, state: int = 4, nseeds: int = 50000) -> dict:
    """Open-loop Poisson arrivals at `rate` per second for `duration` s (SplitMix64(state), seven draws per
    request: exponential gap, Zipf(1.1) rank over nseeds seeds (drawn from SplitMix64(state + 100)), then
    version, dimension, side, x, z as in the uneven batch).  Returns arrays: t (arrival, s), seed, version
    and dimension (indices into C4_VERSIONS and C4_DIMS), side, qx0, qz0 (quart cells), qy."""
    seeds = splitmix64(state + 100, nseeds).view(np.int64)
    cdf = zipf_table(nseeds)
    est = int(rate * duration * 1.2) + 64
    r = splitmix64(state, 7 * est).reshape(est, 7)
    unit = lambda c: (r[:, c] >> np.uint64(11)).astype(np.float64) * 2.0 ** -53  # noqa: E731
    t = np.cumsum(-np.log1p(-unit(0)) / rate)
    n = int(np.searchsorted(t, duration, side="left"))
    rank = np.minimum(np.searchsorted(cdf, unit(1), side="right"), nseeds - 1)
    side = np.floor(16.0 * np.power(32.0, unit(4))).astype(np.int64)
    x = -30000 + (r[:, 5] % np.uint64(60001)).astype(np.int64)
    z = -30000 + (r[:, 6] % np.uint64(60001)).astype(np.int64)
    return {"t": t[:n], "seed": seeds[rank[:n]], "version": (r[:n, 2] % np.uint64(3)).astype(np.int64),
            "dim": (r[:n, 3] % np.uint64(10)).astype(np.int64), "side": side[:n], "qx0": x[:n] >> 2,
            "qz0": z[:n] >> 2, "qy": 16}


def stream_request(stream: dict, i: int):
    """Request i of a stream as (version, dimension, seed, qx0, qz0, side, qy)."""
    return (C4_VERSIONS[stream["version"][i]], C4_DIMS[stream["dim"][i]], int(stream["seed"][i]),
            int(stream["qx0"][i]), int(stream["qz0"][i]), int(stream["side"][i]), stream["qy"])


def serve_run(mg, worlds, stream, budget: int, max_inflight: int = 2, keep_every: int = 0):
    """Replay an arrival stream against a server with the library's native open-loop load generator
    (mcgen_gb300_server_replay: a native submitter thread keeps the schedule, latency runs from each request's
    scheduled arrival).  Ids go to a ring of output slots; with keep_every > 0 every keep_every-th request
    gets a slot of its own and its ids are returned for a parity check."""
    n = len(stream["t"])
    keys = [(v, d) for v in C4_VERSIONS for d in C4_DIMS]
    uniq = sorted(set(keys))
    wlist = [worlds[k] for k in uniq]
    kidx = np.array([uniq.index((C4_VERSIONS[v], C4_DIMS[d])) for v in range(3) for d in range(10)], np.int64)
    widx = kidx[stream["version"] * 10 + stream["dim"]]
    side = stream["side"]
    reqs = mg.RequestArray.from_index(wlist, widx, stream["seed"], stream["qx0"], stream["qz0"], side, side,
                                      stream["qy"])
    slot, ring = 512 * 512, 2048
    kept_idx = np.arange(0, n, keep_every) if keep_every else np.zeros(0, np.int64)
    off = (np.arange(n) % ring) * slot
    off[kept_idx] = (ring + np.arange(kept_idx.size)) * slot
    out = np.empty((ring + kept_idx.size) * slot, np.uint8)
    srv = mg.Server(hbm_budget_bytes=budget, max_inflight=max_inflight)
    lat, elapsed = srv.replay(reqs, stream["t"], out, off)
    st = srv.stats()
    srv.close()
    samples = int((side * side).sum())
    looks = st["cache_hits"] + st["cache_misses"]
    res = {"requests": n, "elapsed_s": round(elapsed, 3), "achieved_rps": round(n / elapsed, 1),
           "samples_per_s": samples / elapsed, "p50_ms": round(float(np.percentile(lat, 50)), 3),
           "p99_ms": round(float(np.percentile(lat, 99)), 3), "max_ms": round(float(lat.max()), 3),
           "latency_from": "scheduled arrival (native open-loop submitter)",
           "cache_hit_rate": round(st["cache_hits"] / max(1, looks), 4), "cache_evictions": st["cache_evictions"],
           "batches": st["batches"], "mean_batch": round(st["requests_admitted"] / max(1, st["batches"]), 2)}
    if not keep_every:
        return res
    kept = [(int(i), out[off[i]:off[i] + side[i] * side[i]].reshape(side[i], side[i]).copy()) for i in kept_idx]
    return res, kept


def serve_parity(stream, kept) -> tuple[dict, dict]:
    """The reference algorithm (oracle port) on all host cores over the kept served requests, timed (the CPU
    baseline of the stream) and compared with the ids the server returned (parity)."""
    import __graft_entry__ as ge
    from oracle import oracle as O

    cores = os.cpu_count() or 1
    wl, mism, cmp_, dt = {}, 0, 0, 0.0
    for i, ids in kept:
        v, d, s, qx0, qz0, n, qy = stream_request(stream, i)
        if (v, d) not in wl:
            wl[(v, d)] = O.World(ge.data_root(), v, d.split(":")[1])
        t0 = time.perf_counter()
        exp = wl[(v, d)].quart_grid(s, qx0, qz0, n, n, qy, O.TIE_ENGINE, threads=cores)
        dt += time.perf_counter() - t0
        mism += int(np.count_nonzero(ids != exp))
        cmp_ += n * n
    base = {"value": cmp_ / max(dt, 1e-9), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{len(kept)} requests at a fixed stride of the stream ({cmp_} samples, {dt:.1f} s), rows over "
                      "threads"}
    parity = {"against": ORACLE_NOTE, "requests": len(kept), "compared_samples": cmp_, "mismatches": mism,
              "sample": "a fixed stride of the served requests, their ids as the server returned them"}
    return base, parity


SEARCH_SEED = 8675309


def search_fixture_rows():
    """(qx, qy, qz, [biome names]) of the reference's known-answer file for seed 8675309 (a test fixture)."""
    rows = []
    path = os.path.join(REPO, "tests", "golden", "search", f"example_obs_26.3_overworld_seed{SEARCH_SEED}.txt")
    for ln in open(path):
        if ln.startswith("#") or not ln.strip():
            continue
        x, y, z, b = ln.split()
        rows.append((int(x), int(y), int(z), b.split("|")))
    return rows


def search_observations(mg, ge, version: str, dim: str):
    """Observations of seed 8675309: the reference's 8-cell Overworld 26.3 known-answer file (committed as a
    fixture) for the Overworld; for the Nether and the End, 8 cells at SplitMix64(5) positions in
    [-5000, 5000) quarts with the biomes this library computes for that seed."""
    if dim == "minecraft:overworld":
        names = {n: i for i, n in enumerate(mg.Generator.open(ge.data_root(), version).biome_names())}
        return mg.make_obs([(x, y, z, [names[n] for n in b]) for x, y, z, b in search_fixture_rows()])
    r = splitmix64(5, 16)
    pts = (-5000 + (r % np.uint64(10000)).astype(np.int64)).reshape(8, 2)
    q = np.stack([pts[:, 0], np.full(8, 16), pts[:, 1]], 1).astype(np.int32)
    w = mg.Generator.open(ge.data_root(), version).world(dim, "normal", 0)
    ids = w.seed_points(np.array([SEARCH_SEED], np.int64), q)[0]
    obs = mg.make_obs([(int(a), int(b), int(c), [int(i)]) for (a, b, c), i in zip(q, ids)])
    if dim == "minecraft:the_end":
        for o in obs:
            o["flags"] = w.end_radius(o["mask"])
    return obs


def run_search(args, rank, world, local_rank, mg, ge):
    """Biome seed search: the range [-2^25, 2^25) of candidate seeds (containing 8675309) against 8
    observations, Overworld 26.3 (the headline value), 26.1, Nether 26.3 and End 26.3; ties mode on."""
    import torch

    torch.cuda.set_device(local_rank)
    n = args.search_candidates
    base = -(n // 2)
    cases = [("26.3", "minecraft:overworld"), ("26.1", "minecraft:overworld"), ("26.3", "minecraft:the_nether"),
             ("26.3", "minecraft:the_end")]
    res = {}
    with ClockSampler(local_rank) as clk:
        for v, d in cases:
            obs = search_observations(mg, ge, v, d)
            w = mg.Generator.open(ge.data_root(), v).world(d, "normal", 0)
            for _ in range(args.warmup):
                w.search(obs, kind=mg.SEEDS_RANGE, base=base, n=1 << 20)
            mg.profile(True)
            dev_ms, wall = 0.0, 0.0
            for _ in range(args.steps):
                t0 = time.perf_counter()
                found, reached, ms = w.search(obs, kind=mg.SEEDS_RANGE, base=base, n=n)
                wall += time.perf_counter() - t0
                dev_ms += ms
            mg.profile(False)
            prof = mg.profile_read()
            res[f"{v} {d.split(':')[1]}"] = {
                "candidates_per_s": n * args.steps / (dev_ms * 1e-3), "e2e_candidates_per_s": n * args.steps / wall,
                "ms_per_step": dev_ms / args.steps, "found": [int(x) for x in found[:8]], "n_found": int(len(found)),
                "reached": [int(x) for x in reached],
                "kernels": {k: {"ms_total": round(a, 3), "launches": b} for k, (a, b) in prof.items()}}
    top = res["26.3 overworld"]
    out = {"metric": "biome seed search candidates/sec", "value": top["candidates_per_s"], "unit": "candidates/s",
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": top["ms_per_step"],
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64+int64",
           "data": "synthetic range of candidate seeds; observations of seed 8675309",
           "config": {"workload": f"seed search: {n} candidates [-{n // 2}, {n // 2}) x 8 observations of seed "
                                  "8675309 (Overworld: the reference's known-answer cells), ties mode",
                      "candidates": n, "cases": res},
           "e2e": {"value": top["e2e_candidates_per_s"], "unit": "candidates/s", "h2d_bytes_per_step": 8 * 32,
                   "d2h_bytes_per_step": 8 * 9 + 8 * top["n_found"]},
           "gpu_launches": sum(v["launches"] for v in top["kernels"].values())}
    clocks = clk.summary()
    if clocks:
        out["clocks"] = clocks
    if rank == 0:
        if not args.skip_extras:
            out["cpu_baseline"] = cpu_baseline_search(mg, ge, args.cpu_sample_s)
    return out


def cpu_baseline_search(mg, ge, budget_s: float) -> dict:
    """The search's reference algorithm (oracle restatement) on all host cores, Overworld 26.3."""
    from oracle import oracle as O

    cores = os.cpu_count() or 1
    obs = O.make_obs([(x, y, z, [O.lib().or_biome_id(n.encode()) for n in b]) for x, y, z, b in search_fixture_rows()])
    w = O.World(ge.data_root(), "26.3", "overworld")
    n = 1 << 14
    while True:
        t0 = time.perf_counter()
        w.search(obs, O.SEEDS_RANGE, base=SEARCH_SEED - n // 2, n=n, threads=cores)
        dt = time.perf_counter() - t0
        if dt > budget_s / 4 or n >= 1 << 24:
            break
        n *= 4
    return {"value": n / dt, "unit": "candidates/s", "cores": cores, "kind": "port",
            "sample": f"{n} candidates around 8675309 ({dt:.2f} s)"}


# The reference's published GPU biome-map times on an RTX 4080 SUPER, 2048 x 2048 cells at step 4 around the
# origin, seed 12345, y = 64, result copied to the host included (docs/blender/gpu.md:116-121, measured with
# libmcgen/tests/g9_bench.c:46-54): seconds per (version, dimension).
MAP2048_PUBLISHED_S = {
    ("26.1", "overworld"): 0.120, ("26.1", "the_nether"): 0.023, ("26.1", "the_end"): 0.079,
    ("26.2", "overworld"): 0.119, ("26.2", "the_nether"): 0.023, ("26.2", "the_end"): 0.074,
    ("26.3", "overworld"): 0.053, ("26.3", "the_nether"): 0.009, ("26.3", "the_end"): 0.074,
    ("26.4-snapshot-2", "overworld"): 0.045, ("26.4-snapshot-2", "the_nether"): 0.009,
    ("26.4-snapshot-2", "the_end"): 0.083}


def run_map(args, rank, world, local_rank, mg, ge):
    """The drop-in biome map: mcgen_gpu_biome_grid(w, -4096, -4096, 2048, 2048, 4, 64, host out) for seed
    12345, every version and dimension (BiomeManager zoom + chunk-cell ties, ids copied to the host), the
    reference's own GPU benchmark shape; best of --steps calls after --warmup."""
    import torch

    torch.cuda.set_device(local_rank)
    n, step, x0 = 2048, 4, -2048 * 4 // 2
    L = mg.load()
    h_out = torch.empty(n * n, dtype=torch.uint8).pin_memory()
    ptr = h_out.data_ptr()
    res = {}
    launches0 = mg.launch_count()
    with ClockSampler(local_rank) as clk:
        for (v, d), pub in MAP2048_PUBLISHED_S.items():
            w = mg.Generator.open(ge.data_root(), v).world("minecraft:" + d, "normal", 12345)
            best = 1e30
            for i in range(args.warmup + args.steps):
                t0 = time.perf_counter()
                rc = L.mcgen_gpu_biome_grid(w.handle, x0, x0, n, n, step, 64, ptr)
                dt = time.perf_counter() - t0
                if rc:
                    raise mg.McError(rc, "mcgen_gpu_biome_grid failed")
                if i >= args.warmup:
                    best = min(best, dt)
            res[f"{v} {d}"] = {"s": round(best, 5), "cells_per_s": n * n / best, "published_4080_s": pub,
                               "speedup_vs_published": round(pub / best, 2)}
    top = res["26.3 overworld"]
    out = {"metric": "biome map cells/sec (mcgen_gpu_biome_grid, ids on the host)", "value": top["cells_per_s"],
           "unit": "cells/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": top["s"] * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": round(top["cells_per_s"] / (n * n / MAP2048_PUBLISHED_S[("26.3", "overworld")]), 3),
           "dtype": "f32+f64+int64", "data": "seed 12345, the reference benchmark's map",
           "config": {"workload": "drop-in biome map 2048 x 2048 cells, x,z in [-4096, 4096) step 4, y=64, seed 12345, "
                                  "zoom + chunk-cell ties, ids copied to pinned host memory; best of steps; "
                                  "vs_baseline against the reference's RTX 4080 SUPER time for Overworld 26.3",
                      "cases": res},
           "e2e": {"value": top["cells_per_s"], "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": n * n},
           "gpu_launches": int(mg.launch_count() - launches0)}
    clocks = clk.summary()
    if clocks:
        out["clocks"] = clocks
    if rank == 0:
        if not args.skip_extras:
            out["cpu_baseline"] = cpu_baseline_map(args.cpu_sample_s)
    return out


def cpu_baseline_map(budget_s: float) -> dict:
    """The oracle's biome map (Overworld 26.3) on all host cores over the first rows of the same map."""
    import __graft_entry__ as ge
    from oracle import oracle as O

    cores = os.cpu_count() or 1
    w = O.World(ge.data_root(), "26.3", "overworld")
    rows = 8
    while True:
        t0 = time.perf_counter()
        w.biome_grid(12345, -4096, -4096, 2048, rows, 4, 64, threads=cores)
        dt = time.perf_counter() - t0
        if dt > budget_s / 4 or rows >= 2048:
            break
        rows = min(2048, rows * 4)
    return {"value": 2048 * rows / dt, "unit": "cells/s", "cores": cores, "kind": "port",
            "sample": f"{rows} of the 2048 map rows ({dt:.2f} s), rows over threads"}


def run_dims(args, rank, world, local_rank, mg, ge):
    """Other dimensions: 4,096 SplitMix64(2) seeds, a 64 x 64 quart grid at y=64 per seed, Nether 26.3 and
    End 26.3, each dimension one batched launch (plan + graph) of 4,096 requests."""
    import torch

    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    seeds, origins = config3_inputs()
    gen = mg.Generator.open(ge.data_root(), "26.3")
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    res = {}
    total_samples, total_ms, kern = 0, 0.0, {}
    total_e2e_s, total_h2d = 0.0, 0
    outs = {}
    with ClockSampler(local_rank) as clk:
        for dim in ("minecraft:the_nether", "minecraft:the_end"):
            w = gen.world(dim, "normal", 0)
            plan = mg.Plan([(w, int(s), int(qx), int(qz), 64, 64, 16) for s, (qx, qz) in zip(seeds, origins)])
            d_out = torch.empty(plan.output_bytes, dtype=torch.uint8, device=dev)
            plan.autotune(d_out.data_ptr(), reps=1)
            for _ in range(args.warmup):
                plan.run_dev(d_out.data_ptr(), sh)
            torch.cuda.synchronize(dev)
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            for _ in range(args.steps):
                plan.run_dev(d_out.data_ptr(), sh)
            ev1.record(stream)
            torch.cuda.synchronize(dev)
            ms = ev0.elapsed_time(ev1) / args.steps
            outs[dim.split(":")[1]] = d_out.cpu().numpy().reshape(len(seeds), 64, 64)  # request i at offset 4096 i
            mg.profile(True)
            plan.run_dev(d_out.data_ptr(), sh, graph=False)
            torch.cuda.synchronize(dev)
            mg.profile(False)
            for k, v in mg.profile_read().items():
                kern[f"{dim.split(':')[1]}:{k}"] = {"ms_total": round(v[0], 4), "launches": v[1]}
            # end to end: a plan from the host request list, run into pinned host memory, freed -- per step
            h_out = torch.empty(plan.output_bytes, dtype=torch.uint8).pin_memory().numpy()
            seeds_np, qx_np, qz_np = seeds, origins[:, 0], origins[:, 1]
            e2e_steps = 0 if args.skip_extras else min(args.steps, 5)
            t0 = time.perf_counter()
            h2d = 0
            for _ in range(e2e_steps):
                p = mg.Plan(mg.RequestArray(w, seeds_np, qx_np, qz_np, 64, 64, 16))
                p.shape = plan.shape
                p.run(h_out)
                h2d = p.h2d_bytes
                p.close()
            e2e_s = time.perf_counter() - t0
            res[dim.split(":")[1]] = {"ms_per_step": round(ms, 4), "samples_per_s": plan.output_bytes / (ms * 1e-3),
                                      "e2e_samples_per_s": plan.output_bytes * e2e_steps / e2e_s if e2e_steps else None,
                                      "h2d_bytes_per_step": int(h2d), "tile_shape": plan.shape}
            total_samples += plan.output_bytes
            total_ms += ms
            total_e2e_s += e2e_s / e2e_steps if e2e_steps else 0.0
            total_h2d += int(h2d)
    out = {"metric": METRIC, "value": total_samples * world / (total_ms * 1e-3), "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (SplitMix64(2) seeds)",
           "config": {"workload": "other dimensions 26.3: 4096 SplitMix64(2) seeds x 64x64 quart grid at y=64, "
                                  "corners SplitMix64(102) uniform in [-30000,30000) blocks, Nether and End, one "
                                  "batched launch per dimension", "per_dimension": res},
           "kernels": kern, "gpu_launches": args.steps * 4}
    if not args.skip_extras:
        out["e2e"] = {"value": total_samples * world / total_e2e_s, "unit": UNIT, "h2d_bytes_per_step": total_h2d,
                      "d2h_bytes_per_step": int(total_samples),
                      "call": "Plan(RequestArray(world, seeds, corners, 64, 64, 16)) + plan_run(host buffer) + "
                              "plan_free per dimension per step"}
    clocks = clk.summary()
    if clocks:
        out["clocks"] = clocks
    if rank == 0:
        if not args.skip_extras:
            out["cpu_baseline"], out["parity"] = cpu_baseline_dims(args.cpu_sample_s, outs)
    return out


def cpu_baseline_dims(budget_s: float, got: dict, stride: int = 16) -> tuple[dict, dict]:
    """The reference algorithm (oracle port) on all host cores over every `stride`-th seed of the workload
    (until the time budget is used), and the same outputs as the parity check of the GPU's grids.
    Returns (cpu_baseline, parity)."""
    import __graft_entry__ as ge
    from oracle import oracle as O

    cores = os.cpu_count() or 1
    seeds, origins = config3_inputs()
    wn = O.World(ge.data_root(), "26.3", "the_nether")
    we = O.World(ge.data_root(), "26.3", "the_end")
    done, mism, t0 = 0, 0, time.perf_counter()
    for i in range(0, len(seeds), stride):
        sd, (qx, qz) = int(seeds[i]), origins[i]
        en = wn.quart_grid(sd, int(qx), int(qz), 64, 64, 16, O.TIE_ENGINE, threads=cores)
        ee = we.quart_grid(sd, int(qx), int(qz), 64, 64, 16, O.TIE_ENGINE, threads=cores)
        mism += int(np.count_nonzero(got["the_nether"][i] != en)) + int(np.count_nonzero(got["the_end"][i] != ee))
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return ({"value": done * 2 * 64 * 64 / dt, "unit": UNIT, "cores": cores, "kind": "port",
             "sample": f"every {stride}th of the 4096 seeds ({done} seeds), Nether and End ({dt:.1f} s), rows over "
                       "threads"},
            {"against": ORACLE_NOTE, "compared_samples": done * 2 * 64 * 64, "mismatches": mism,
             "sample": f"every {stride}th seed's Nether and End grids (the CPU baseline's outputs)"})


def run_serve(args, rank, world, local_rank, mg, ge):
    """Serving: open-loop Poisson streams at each rate of --rates for --duration s, continuous batching,
    8 GB noise-state cache; latency from each request's scheduled arrival.  With small_budget, one more run at
    the middle rate with a 2 MB cache forces LRU evictions."""
    import torch

    torch.cuda.set_device(local_rank)
    gens = {v: mg.Generator.open(ge.data_root(), v) for v in C4_VERSIONS}
    worlds = {(v, d): gens[v].world(d, "normal", 0) for v in C4_VERSIONS for d in set(C4_DIMS)}
    warm = config5_stream(200.0, 1.0, state=99)
    serve_run(mg, worlds, warm, 8 << 30, args.inflight)
    rates = [float(x) for x in args.rates.split(",")]
    runs = {}
    with ClockSampler(local_rank) as clk:
        for k, rate in enumerate(rates):
            stream = config5_stream(rate, args.duration)
            if k == len(rates) - 1 and not args.skip_extras:
                runs[str(int(rate))], kept = serve_run(mg, worlds, stream, 8 << 30, args.inflight,
                                                       keep_every=max(1, len(stream["t"]) // 200))
                top_stream = stream
            else:
                runs[str(int(rate))] = serve_run(mg, worlds, stream, 8 << 30, args.inflight)
        small = (serve_run(mg, worlds, config5_stream(rates[len(rates) // 2], args.duration / 2), 2 << 20, args.inflight)
                 if getattr(args, "small_budget", True) else None)
    top = runs[str(int(rates[-1]))]
    under = [r for r in rates if runs[str(int(r))]["p99_ms"] < 20.0]
    out = {"metric": METRIC + " (served)", "value": top["samples_per_s"], "unit": UNIT, "n_gpus": world,
           "steps": len(rates), "warmup": 1, "ms_per_step": top["elapsed_s"] * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64+int64",
           "data": "synthetic (SplitMix64(4) Poisson stream, Zipf(1.1) over 50,000 seeds)",
           "config": {"workload": f"served: open-loop Poisson arrivals at {args.rates} req/s for {args.duration} s each, "
                                  "requests from the uneven-batch distribution, seeds Zipf(1.1) over 50,000; "
                                  f"continuous batching on {args.inflight} streams, 8 GB noise-state cache (LRU); "
                                  "latency from scheduled arrival",
                      "rates": rates, "duration_s": args.duration,
                      "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
           "served": runs, "p50_ms": top["p50_ms"], "p99_ms": top["p99_ms"],
           "highest_rate_p99_under_20ms": max(under) if under else None,
           "e2e": {"value": top["samples_per_s"], "unit": UNIT, "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": int(top["samples_per_s"] * top["elapsed_s"]),
                   "call": "mcgen_gb300_server_submit (host output buffer) + server_wait per request"}}
    if small is not None:
        out["small_budget_2MB"] = small
    clocks = clk.summary()
    if clocks:
        out["clocks"] = clocks
    if not args.skip_extras:
        out["cpu_baseline"], out["parity"] = serve_parity(top_stream, kept)
    return out


ORACLE_NOTE = "oracle (the reference engine's CPU algorithm restated, pinned to the reference's golden vectors)"


def cpu_baseline(workload: str, budget_s: float, got: np.ndarray) -> tuple[dict, dict]:
    """The reference algorithm on this host's cores (CPU oracle, OpenMP over seeds or rows) over a sample of
    the workload, and the same outputs as the parity check of the GPU's output `got`.
    Returns (cpu_baseline, parity)."""
    import __graft_entry__ as ge
    from oracle import oracle as O

    cores = os.cpu_count() or 1
    w = O.World(ge.data_root(), "26.3", "overworld")
    if workload == "seeds8":
        seeds, pts = config2_inputs(got.size // 8)
        got = got.reshape(seeds.size, len(pts))
        stride = 256
        while True:  # a stride sample of the seeds, grown until it takes a meaningful share of the budget
            t0 = time.perf_counter()
            exp = w.points(seeds[::stride], pts, threads=cores)
            dt = time.perf_counter() - t0
            if dt > budget_s / 4 or stride == 1:
                break
            stride = max(1, stride // 4)
        n = exp.shape[0]
        mism = int(np.count_nonzero(got[::stride] != exp))
        return ({"value": n * len(pts) / dt, "unit": UNIT, "cores": cores, "kind": "port",
                 "sample": f"every {stride}th of the {seeds.size} seeds x 8 points ({n} seeds, {dt:.2f} s)"},
                {"against": ORACLE_NOTE, "compared_samples": int(exp.size), "mismatches": mism,
                 "sample": f"every {stride}th seed x 8 points (the CPU baseline's outputs)"})
    t0 = time.perf_counter()
    exp = w.biome_grid(12345, -512, -512, 256, 256, 4, 64, threads=cores)
    dt = time.perf_counter() - t0
    mism = int(np.count_nonzero(got.reshape(256, 256) != exp))
    return ({"value": 256 * 256 / dt, "unit": UNIT, "cores": cores, "kind": "port",
             "sample": f"the whole 256 x 256 grid ({dt:.2f} s), rows over threads"},
            {"against": ORACLE_NOTE, "compared_samples": 256 * 256, "mismatches": mism,
             "sample": "the whole drop-in grid (zoom + chunk-cell ties)"})


# FNV-1a64 digest of the reference's golden 1024 x 1024 quart grid (GRID_CHAIN ties) of Overworld 26.3,
# seed 12345, qx, qz in [-512, 512), qy = 16 (tests/vectors/26.3/biome_grid_hashes.tsv, mode "point")
C1_GOLDEN_DIGEST = "a79bc97b2afa0ecd"


def quart_form_parity(mg, gen, dev) -> dict:
    """C1's quart form: the 256 x 256 quart grid qx, qz in [-128, 128) at qy = 16 (ENGINE ties) through
    mcgen_gb300_quart_grid against the oracle, and its 1024 x 1024 superset under GRID_CHAIN against the
    reference's golden digest."""
    import __graft_entry__ as ge
    from oracle import oracle as O

    w = gen.world("minecraft:overworld", "normal", 12345)
    got = w.quart_grid(-128, -128, 256, 256, 16, mg.TIE_ENGINE)
    exp = O.World(ge.data_root(), "26.3", "overworld").quart_grid(12345, -128, -128, 256, 256, 16, O.TIE_ENGINE)
    big = w.quart_grid(-512, -512, 1024, 1024, 16, mg.TIE_GRID_CHAIN)
    digest = O.fnv1a64_names(big)
    return {"against": ORACLE_NOTE + "; the golden digest", "compared_samples": 256 * 256,
            "mismatches": int(np.count_nonzero(got != exp)), "golden_digest_1024": digest,
            "golden_digest_match": digest == C1_GOLDEN_DIGEST}


def quart_form_rate(mg, gen, dev, steps: int, warmup: int) -> dict:
    """C1's quart form timed: the 256 x 256 quart grid qx, qz in [-128, 128) at qy = 16 (ENGINE ties) through
    mcgen_gb300_quart_grid_dev (one world, its lattices resident), CUDA events per step with L2 flushed
    between steps; and end to end through mcgen_gb300_quart_grid (host output buffer)."""
    import torch

    w = gen.world("minecraft:overworld", "normal", 12345)
    n = 256 * 256
    d_out = torch.empty(n, dtype=torch.uint8, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(warmup):
        w.quart_grid_dev(-128, -128, 256, 256, 16, mg.TIE_ENGINE, d_out.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize(dev)
    ms = 0.0
    for _ in range(steps):
        flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        w.quart_grid_dev(-128, -128, 256, 256, 16, mg.TIE_ENGINE, d_out.data_ptr(), stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms += e0.elapsed_time(e1)
    for _ in range(warmup):
        w.quart_grid(-128, -128, 256, 256, 16, mg.TIE_ENGINE)
    t0 = time.perf_counter()
    for _ in range(steps):
        w.quart_grid(-128, -128, 256, 256, 16, mg.TIE_ENGINE)
    e2e_s = time.perf_counter() - t0
    return {"value": n * steps / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms / steps,
            "e2e": {"value": n * steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": n},
            "form": "mcgen_gb300_quart_grid: 256 x 256 quarts qx, qz in [-128, 128), qy = 16, ENGINE ties"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    import __graft_entry__ as ge
    from oracle import oracle as O

    cores = os.cpu_count() or 1
    w = O.World(ge.data_root(), "26.3", "overworld")
    if args.workload == "seeds8":
        seeds, pts = config2_inputs()
        n = 4096
        per_step = lambda: w.points(seeds[:n], pts, threads=cores)  # noqa: E731
        samples = n * len(pts)
        sample = f"first {n} of the 65536 seeds x 8 points per step"
        config = {"workload": "Overworld 26.3 normal, 65536 SplitMix64(1) seeds x 8 fixed points, ENGINE tie rule",
                  "version": "26.3", "dimension": "overworld"}
    elif args.workload in ("batch10k", "serve"):
        reqs = config4_requests(args.requests)
        wl = {}
        classes = {c: [i for i, r in enumerate(reqs) if class_of(r[0], r[1]) == c] for c in BATCH_CLASSES}
        total = {c: sum(reqs[i][5] ** 2 for i in idx) for c, idx in classes.items() if idx}
        stride = 40
        step_no = [0]
        acc = {c: [0, 0.0] for c in total}  # per class: samples, seconds

        def per_step():
            k = step_no[0] % stride
            step_no[0] += 1
            for c in total:
                t0, cells = time.perf_counter(), 0
                for i in classes[c][k::stride]:
                    v, d, s, qx0, qz0, n, qy = reqs[i]
                    if (v, d) not in wl:
                        wl[(v, d)] = O.World(ge.data_root(), v, d.split(":")[1])
                    wl[(v, d)].quart_grid(s, qx0, qz0, n, n, qy, O.TIE_ENGINE, threads=cores)
                    cells += n * n
                acc[c][0] += cells
                acc[c][1] += time.perf_counter() - t0

        def weighted():  # the whole batch's samples over the time the per-class rates give it
            return sum(total.values()) / sum(total[c] / (acc[c][0] / acc[c][1]) for c in total)

        samples = sum(total.values())
        sample = (f"per step every {stride}th request of each code-path class (a different offset each step), rows "
                  "over threads; rate = the whole batch's samples / the sum of its per-class samples over the "
                  "per-class rates")
        config = {"workload": f"uneven mixed batch: {len(reqs)} SplitMix64(3) requests, versions 26.1/26.2/26.3, "
                              "Overworld:Nether:End 6:2:2, square side log-uniform in [16,512) quart cells, origin "
                              "uniform in [-30000,30000] blocks, y=64, ENGINE tie rule", "requests": len(reqs)}
    elif args.workload == "dims4096":
        seeds, origins = config3_inputs()
        wn = O.World(ge.data_root(), "26.3", "the_nether")
        we = O.World(ge.data_root(), "26.3", "the_end")
        nfirst = 16

        def per_step():
            for sd, (qx, qz) in zip(seeds[:nfirst], origins[:nfirst]):
                wn.quart_grid(int(sd), int(qx), int(qz), 64, 64, 16, O.TIE_ENGINE, threads=cores)
                we.quart_grid(int(sd), int(qx), int(qz), 64, 64, 16, O.TIE_ENGINE, threads=cores)

        samples = nfirst * 2 * 64 * 64
        sample = f"first {nfirst} of the 4096 seeds, Nether and End 64x64 grids per step"
        config = {"workload": "other dimensions 26.3: 4096 SplitMix64(2) seeds x 64x64 quart grid at y=64, "
                              "Nether and End"}
    elif args.workload == "search":
        obs = O.make_obs([(x, y, z, [O.lib().or_biome_id(n.encode()) for n in b]) for x, y, z, b in search_fixture_rows()])
        ncand = 1 << 18
        per_step = lambda: w.search(obs, O.SEEDS_RANGE, base=SEARCH_SEED - ncand // 2, n=ncand, threads=cores)  # noqa: E731
        samples = ncand
        sample = f"{ncand} candidates around 8675309 per step, candidates over threads"
        config = {"workload": "seed search: candidates x 8 observations of seed 8675309 (the reference's known-answer "
                              "cells), Overworld 26.3, ties mode"}
    else:
        rows = 32
        per_step = lambda: w.biome_grid(12345, -512, -512, 256, rows, 4, 64, threads=cores)  # noqa: E731
        samples = 256 * rows
        sample = f"{rows} of 256 grid rows per step"
        config = {"workload": "Overworld 26.3 normal, seed 12345, biome grid 256x256 step 4 y=64",
                  "version": "26.3", "dimension": "overworld"}
    metric, unit = (("biome seed search candidates/sec", "candidates/s") if args.workload == "search"
                    else (METRIC, UNIT))
    for _ in range(args.warmup):
        per_step()
    if args.workload in ("batch10k", "serve"):
        for c in acc:
            acc[c] = [0, 0.0]
    t0 = time.perf_counter()
    for _ in range(args.steps):
        per_step()
    dt = time.perf_counter() - t0
    value = samples * args.steps / dt
    full_batch_s = None
    if args.workload in ("batch10k", "serve"):
        value = weighted()
        full_batch_s = samples / value  # the whole batch at the measured per-class rates
    out = {"impl": "reference", "metric": metric, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32+f64+int64", "data": "synthetic (SplitMix64 seeds and points)",
           "config": config,
           "cpu_baseline": {"value": value, "unit": unit, "cores": cores, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if full_batch_s is not None:
        out["full_batch_s"] = round(full_batch_s, 2)
    print(json.dumps(out), flush=True)


# The configurations besides the headline (C4): the plain single-seed grid (C1, drop-in and quart forms),
# many seeds x fixed points (C2), the other dimensions (C3) and the served stream at 2,000 requests/s for
# 60 s (C5), each with its device value, end-to-end value, CPU baseline and parity check.
CONFIGS = (("C1_grid256", "grid256", {}), ("C2_seeds8", "seeds8", {}), ("C3_dims4096", "dims4096", {}),
           ("C5_serve_2000rps_60s", "serve", {"rates": "2000", "duration": 60.0, "small_budget": False}))
CONFIG_KEYS = ("metric", "value", "unit", "ms_per_step", "steps", "config", "e2e", "cpu_baseline", "parity",
               "parity_quart_form", "quart_form", "roofline", "kernels", "gpu_launches", "served", "p50_ms", "p99_ms",
               "highest_rate_p99_under_20ms", "clocks")


def run_configs(args, rank, world, local_rank) -> dict:
    import copy

    res = {}
    for name, workload, extra in CONFIGS:
        sub = copy.copy(args)
        sub.workload = workload
        sub.split_classes = False
        sub.cpu_sample_s = min(args.cpu_sample_s, 6.0)
        sub.seeds = 65536
        for k, v in extra.items():
            setattr(sub, k, v)
        line = run_gb300(sub, rank, world, local_rank)
        res[name] = {k: line[k] for k in CONFIG_KEYS if k in line}
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=["seeds8", "grid256", "batch10k", "serve", "dims4096", "search", "map2048"],
                    default="batch10k")
    ap.add_argument("--search-candidates", type=int, default=1 << 26, help="search: candidates per step")
    ap.add_argument("--rates", default="500,1000,2000", help="serve: arrival rates (requests/s)")
    ap.add_argument("--duration", type=float, default=60.0, help="serve: seconds per rate (60 = the configuration)")
    ap.add_argument("--inflight", type=int, default=2, help="serve: batches in flight (server streams)")
    ap.add_argument("--no-configs", action="store_true",
                    help="batch10k: the headline only, without the other configurations")
    ap.add_argument("--requests", type=int, default=10000, help="batch10k: number of requests")
    ap.add_argument("--class", dest="batch_class", choices=["overworld_double", "overworld_float", "nether_double",
                                                            "nether_float", "end"], default=None,
                    help="batch10k: only the requests of one code-path class (profiling)")
    ap.add_argument("--split-classes", action="store_true",
                    help="batch10k: also time each code-path class's requests as a plan of their own")
    ap.add_argument("--cpu-sample-s", type=float, default=12.0)
    ap.add_argument("--seeds", type=int, default=65536, help="seeds8: number of seeds (65536 = the configuration)")
    ap.add_argument("--skip-extras", action="store_true",
                    help="profiling runs: no e2e pass, no pipe peaks, no CPU baseline")
    args = ap.parse_args()
    rank, world, local_rank = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    try:
        out = run_gb300(args, rank, world, local_rank)
        if args.workload == "batch10k" and not (args.skip_extras or args.no_configs) and world == 1:
            out["configs"] = run_configs(args, rank, world, local_rank)
        if rank == 0 and out is not None:
            print(json.dumps(out), flush=True)
    finally:
        if world > 1:
            import torch

            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
