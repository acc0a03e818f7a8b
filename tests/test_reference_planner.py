"""Which inputs the reference binary can run safely, from a CPU restatement of its planner.

oracle/ref_planner.py restates the reference's host planner (src/utils/util.cu:37-74,
src/simulation/proliferation.cu:26-284): the recursion depth chosen from free device memory,
the level sizes (uint32_t), the grid size (uint16_t) and whether a second iteration starts.
With the deepest generation each input reaches (the oracle's max_gen), it decides which
configured inputs the distribution check and the timing comparison may run on a GPU. Free
memory on a GB300 is about 296 GB; the conclusions hold from 200 GB up.
"""
import pytest

import procell.configs as cfg

FREE = (200e9, 296e9)


@pytest.fixture(scope="module")
def planner():
    import ref_planner
    return ref_planner


def max_gen_and_values(oracle_lib, w, root_end=None):
    o = oracle_lib.simulate(w.bins, w.types, w.t_max, w.phi, seed=w.seed, root_end=root_end, nthreads=0)
    return o.stats["max_gen"], len(o.values)


def test_max_recursion_depth_restatement(planner):
    # the small workload (9512 initial cells, 390 output values) with 200 GB free: the loop
    # of util.cu:55-66 ends 18 doublings up, and 0.9 x 18 truncates to 16
    assert planner.max_recursion_depth(390, 9512, int(200e9)) == 16
    assert planner.max_recursion_depth(0, 10, 100) == 0  # 2 x 400 B > 100 B
    assert planner.max_recursion_depth(0, 1, 10 ** 15) == planner.MAX_DEPTH
    assert planner.n_blocks(9512) == 10 and planner.n_blocks(1023) == 1 and planner.n_blocks(1024) == 2


@pytest.mark.parametrize("free", FREE)
def test_small_runs_in_one_safe_iteration(oracle_lib, planner, free):
    w = cfg.small()
    g, nv = max_gen_and_values(oracle_lib, w)
    a = planner.assess(w.roots, nv, g, int(free), len(w.types))
    assert a["safe"], a["reasons"]
    assert a["depth"] > g and a["n_blocks"] < 2 ** 16 and a["largest_level"] < 2 ** 32


@pytest.mark.parametrize("free", FREE)
def test_medium_histogram_at_t150_runs_in_one_safe_iteration(oracle_lib, planner, free):
    w = cfg.medium()
    w.t_max = 150.0
    g, nv = max_gen_and_values(oracle_lib, w)
    a = planner.assess(w.roots, nv, g, int(free), len(w.types))
    assert a["safe"], a["reasons"]
    assert g == 8 and a["depth"] >= 9


@pytest.mark.parametrize("free", FREE)
def test_medium_histogram_with_shared_timers_runs_in_one_safe_iteration(oracle_lib, planner, free):
    w = cfg.medium()
    w.t_max = 150.0
    w.types = [(0.4, 60.0, 18.0), (0.35, 60.0, 18.0), (0.25, 60.0, 18.0)]
    g, nv = max_gen_and_values(oracle_lib, w)
    a = planner.assess(w.roots, nv, g, int(free), len(w.types))
    assert a["safe"], a["reasons"]


@pytest.mark.parametrize("free", FREE)
@pytest.mark.parametrize("name", ["medium", "large"])
def test_configured_medium_and_large_need_a_second_iteration(oracle_lib, planner, free, name):
    w = cfg.by_name(name)
    # the deepest generation of a prefix of the initial cells is a lower bound for the whole
    g, nv = max_gen_and_values(oracle_lib, w, root_end=None if name == "medium" else w.roots // 200)
    a = planner.assess(w.roots, nv, g, int(free), len(w.types), track_ratio=(name == "medium"))
    assert not a["safe"]
    assert any("second iteration" in r for r in a["reasons"])
    # the second iteration's population is the whole last level: its grid size wraps
    assert planner.n_blocks(a["largest_level"]) >= 2 ** 16
