"""CPU pins of the seed-search restatement (oracle.or_search): the reference's known-answer files --
observations of a known seed from its Java oracle -- must give back exactly that seed among the 2^16
structure-seed candidates (crack/src/gpu_biomes/results/test_b_known_answer.txt: found, 1 passing)."""
import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import oracle as O
from search_cases import example_files, read_example


@pytest.mark.parametrize("path", example_files(), ids=lambda p: p.rsplit("_", 1)[1][:-4])
def test_known_answer_structure_search(path):
    version, dim, seed, rows = read_example(path)
    w = O.World(ge.data_root(), version, dim)
    obs = O.make_obs(rows)
    found, reached = w.search(obs, O.SEEDS_STRUCTURE, base=seed & ((1 << 48) - 1))
    assert list(found) == [seed]
    assert int(reached[-1]) == 1 and int(reached.sum()) == 65536


def test_end_radius_rule():
    """The End window half-width: no class threshold crossed -> 0; islands vs the rest -> the widest."""
    w = O.World(ge.data_root(), "26.3", "the_end")
    ids = {n: O.lib().or_biome_id(n.encode()) for n in ("the_end", "end_highlands", "end_midlands",
                                                         "small_end_islands", "end_barrens")}

    def mask(*names):
        m = np.zeros(2, np.uint64)
        for n in names:
            m[ids[n] >> 6] |= np.uint64(1) << np.uint64(ids[n] & 63)
        return m

    assert w.end_radius(mask("small_end_islands", "end_barrens", "end_midlands", "end_highlands")) == 0
    assert w.end_radius(mask("end_highlands")) == int(((101 - 40) / 9 + 1) / 2)
    assert w.end_radius(mask("small_end_islands")) == min(12, int(((101 + 20) / 9 + 1) / 2))
