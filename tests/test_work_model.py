"""The work model behind the bench's roofline figures, pinned against the oracle's work counter: octave
(lattice) samples per biome sample for every version and dimension."""
import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import oracle as O

VERSIONS = ["26.1", "26.2", "26.3", "26.4-snapshot-2"]


@pytest.mark.parametrize("version", VERSIONS)
@pytest.mark.parametrize("dim", ["overworld", "the_nether"])
def test_octaves_per_sample(version, dim):
    import bench

    rng = np.random.default_rng(5)
    pts = np.stack([rng.integers(-9000, 9000, 32), rng.integers(-16, 80, 32), rng.integers(-9000, 9000, 32)], 1)
    w = O.World(ge.data_root(), version, dim)
    for seed in (1, -77, 2**62 + 3):
        work = w.work(seed, pts)
        assert work["octave_samples"] == len(pts) * bench.OCTAVES_PER_SAMPLE["minecraft:" + dim]
        assert work["tree_queries"] == len(pts)


def test_fp64_model_covers_versions():
    import bench

    reqs = [("26.1", "minecraft:overworld", 1, 0, 0, 16, 16), ("26.3", "minecraft:the_nether", 2, 0, 0, 8, 16),
            ("26.2", "minecraft:the_end", 3, 0, 0, 16, 16), ("26.4-snapshot-2", "minecraft:overworld", 4, 0, 0, 2, 16),
            ("26.2", "minecraft:the_nether", 5, 0, 0, 4, 16)]
    assert bench.batch_fp64_ops(reqs) == 256 * 446 + 64 * 8 * 2 + 0 + 4 * 52 * 2 + 16 * 16
    # the double branch's model: 12 shift octave samples in double with tabled splits and smoothsteps, the
    # per-tile table (6 x 48 entries of 8 over 128 cells), 40 fixed-point ones (screens off the FP64 pipe)
    assert bench.FP64_PER_SAMPLE[("double", "minecraft:overworld")] == 12 * 29 + 6 * 48 * 8 // 128 + 40 * 2
    assert bench.FP64_PER_SAMPLE[("float", "minecraft:overworld")] == bench.OCTAVES_PER_SAMPLE["minecraft:overworld"] * 2
