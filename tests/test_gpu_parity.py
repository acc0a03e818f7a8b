"""GPU parity: the sm_103a engine against the CPU oracle, bit-exact.

Every case runs the engine through the C ABI (libprocell.so via ctypes) and the oracle on
the same inputs and seed, and requires identical uint64 histograms, per-type columns and
statistics. Cases follow the reference's rules and edge cases (src/io/parser.cu:68-217,
src/simulation/cell.cu:25-143, src/simulation/proliferation.cu:289-410).
"""
import numpy as np
import pytest

import procell.configs as cfg

pytestmark = pytest.mark.gpu


def both(engine, oracle_lib, bins, types, t_max, phi, seed, **kw):
    g = engine.simulate(bins, types, t_max, phi, seed, **kw)
    o = oracle_lib.simulate(bins, types, t_max, phi, seed=seed,
                            root_begin=kw.get("root_begin") or 0,
                            root_end=kw.get("root_end"), nthreads=0)
    return g, o


def assert_same(g, o):
    assert np.array_equal(g.values, o.values)
    assert np.array_equal(g.totals, o.totals), (np.flatnonzero(g.totals != o.totals)[:10])
    assert np.array_equal(g.per_type, o.per_type)
    for k in ("roots", "divisions", "leaves", "uncounted", "vanished"):
        assert g.stats[k] == o.stats[k], (k, g.stats[k], o.stats[k])
    assert g.stats["max_generation"] == o.stats["max_gen"]


def test_philox_device_matches_oracle(engine, oracle_lib):
    rng = np.random.default_rng(1)
    ctr = rng.integers(0, 2 ** 32, size=(4096, 4), dtype=np.uint64).astype(np.uint32)
    ctr[0] = 0
    ctr[1] = 0xFFFFFFFF
    key = [0xA4093822, 0x299F31D0]
    dev = engine.philox(ctr, key)
    for i in range(0, 4096, 97):
        assert list(dev[i]) == oracle_lib.philox(list(map(int, ctr[i])), key)
    assert list(engine.philox(np.array([[0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344]]),
                              [0xA4093822, 0x299F31D0])[0]) == [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_tables_match_oracle(engine, oracle_lib):
    for a, b in zip(engine.tables(), oracle_lib.tables()):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_normals_device_matches_oracle(engine, oracle_lib):
    z = engine.normals(seed=77, root=12345, first_parent=1 << 20, count=300_000)
    o = oracle_lib.normals(seed=77, root=12345, first_parent=1 << 20, count=300_000)
    assert np.array_equal(z.view(np.uint32), o.view(np.uint32))


def test_small_config_bit_exact(engine, oracle_lib):
    w = cfg.small()
    g, o = both(engine, oracle_lib, w.bins, w.types, w.t_max, w.phi, w.seed)
    assert_same(g, o)
    assert g.stats["divisions"] > 10_000


def test_medium_config_bit_exact(engine, oracle_lib):
    w = cfg.medium()
    g, o = both(engine, oracle_lib, w.bins, w.types, w.t_max, w.phi, w.seed)
    assert_same(g, o)


@pytest.mark.parametrize("seed", [0, 1, 2 ** 63 + 5])
def test_seeds(engine, oracle_lib, seed):
    w = cfg.small(seed=5)
    g, o = both(engine, oracle_lib, w.bins, w.types, w.t_max, w.phi, seed)
    assert_same(g, o)


def test_large_root_subsample_bit_exact(engine, oracle_lib):
    w = cfg.large()
    n = w.roots
    g, o = both(engine, oracle_lib, w.bins, w.types, w.t_max, w.phi, w.seed,
                root_begin=n // 2, root_end=n // 2 + n // 200)
    assert_same(g, o)


EDGE_CASES = {
    "empty": ([], [(1.0, 10.0, 1.0)], 50.0, 1.0),
    "all_zero_freq": ([(3.0, 0), (5.0, 0)], [(1.0, 10.0, 1.0)], 50.0, 1.0),
    "single_root": ([(1000.0, 1)], [(1.0, 10.0, 3.0)], 100.0, 1.0),
    "quiescent_only": ([(8.0, 3), (1.0, 5), (0.5, 2)], [(1.0, -1.0, -1.0)], 100.0, 1.0),
    "t_max_zero": ([(64.0, 50), (3.0, 20)], [(0.5, 10.0, 2.0), (0.5, 20.0, 1.0)], 0.0, 1.0),
    "sd_zero": ([(64.0, 4000)], [(1.0, 10.0, 0.0)], 15.0, 1.0),
    "mean_zero": ([(64.0, 40), (10.0, 5)], [(0.5, 0.0, 1.0), (0.5, 5.0, 1.0)], 30.0, 1.0),
    "phi_boundary": ([(2.0, 100), (2.0 + 2 ** -40, 10)], [(1.0, 1.0, 0.1)], 1e6, 1.0),
    "heavy_truncation": ([(4096.0, 300)], [(1.0, 1.0, 3.0)], 12.0, 1.0),
    "negative_sd": ([(512.0, 500)], [(0.7, 20.0, -6.0), (0.3, 30.0, 9.0)], 120.0, 1.0),
    "duplicate_values": ([(16.0, 30), (16.0, 20), (8.0, 40)], [(1.0, 5.0, 1.0)], 40.0, 1.0),
    "below_phi_roots": ([(0.5, 30), (0.9, 7), (20.0, 9)], [(0.5, 4.0, 1.0), (0.5, -1.0, -1.0)], 30.0, 1.0),
    "auto_phi": ([(5.0, 0), (3.0, 20), (700.0, 10)], [(1.0, 6.0, 2.0)], 60.0, None),
    "many_types": ([(1e4, 2000)], [(1.0 / 7, 5.0 + i, 1.0 + 0.3 * i) for i in range(7)], 60.0, 1.0),
    "ratio_ties": ([(300.0, 3000)], [(0.25, 10.0, 3.0), (0.25, 20.0, 3.0), (0.5, 15.0, 2.0)], 80.0, 1.0),
    "zero_ratio_type": ([(300.0, 3000)], [(0.0, 10.0, 3.0), (1.0, 20.0, 3.0)], 80.0, 1.0),
    "deep_tree": ([(2.0 ** 40, 3)], [(1.0, 1.0, 0.05)], 30.0, 1.0),
    # phi cap exactly 32 and lineages through generation 31: the daughters of generation-31
    # cells (generation 32, never stored) are parked with a key when their first draw is
    # not settled, so keys of generation 32 must fit the layout (about 1e7 divisions)
    "narrow_boundary": ([(2.0 ** 32.5, 3)], [(1.0, 1.0, 0.5)], 22.0, 1.0),
    "tiny_phi": ([(1e-3, 50)], [(1.0, 2.0, 0.4)], 24.0, 1e-9),
    "huge_t": ([(1e5, 200)], [(1.0, 3.0, 1.0)], 1e9, 1.0),
}


@pytest.mark.parametrize("name", sorted(EDGE_CASES))
def test_edge_cases(engine, oracle_lib, name):
    bins, types, t, phi = EDGE_CASES[name]
    g, o = both(engine, oracle_lib, bins, types, t, phi, 12345)
    assert_same(g, o)


def test_results_independent_of_chunking_and_grid(engine, oracle_lib):
    w = cfg.medium()
    base = engine.simulate(w.bins, w.types, w.t_max, w.phi, w.seed)
    try:
        engine.set_option("max_slice_cells", 100_003)
        engine.set_option("max_root_chunk", 77_777)
        engine.set_option("grid_blocks", 37)
        other = engine.simulate(w.bins, w.types, w.t_max, w.phi, w.seed)
    finally:
        engine.set_option("max_slice_cells", 0)
        engine.set_option("max_root_chunk", 0)
        engine.set_option("grid_blocks", 0)
    assert np.array_equal(base.per_type, other.per_type)
    assert base.stats["divisions"] == other.stats["divisions"]
    assert other.stats["sweeps"] > base.stats["sweeps"]


def test_shards_add_up(engine):
    w = cfg.small()
    full = engine.simulate(w.bins, w.types, w.t_max, w.phi, w.seed)
    n = w.roots
    cuts = [0, 1, n // 3, n // 2, n - 1, n]
    parts = [engine.simulate(w.bins, w.types, w.t_max, w.phi, w.seed, root_begin=a, root_end=b)
             for a, b in zip(cuts, cuts[1:])]
    assert np.array_equal(sum(p.per_type for p in parts), full.per_type)
    assert sum(p.stats["divisions"] for p in parts) == full.stats["divisions"]


@pytest.mark.parametrize("name", ["medium", "edge"])
def test_device_and_host_merge_agree(engine, oracle_lib, name):
    """pc_plan_result merges the counts into the value histogram on the device and reads back
    only the merged counts; the host merge (used for plans whose merge scratch would exceed
    256 MB, forced here by the option device_merge = 0) must give the same histogram, and
    both the oracle's."""
    if name == "medium":
        w = cfg.medium()
        bins, types, t_max, phi, seed = w.bins, w.types, w.t_max, w.phi, w.seed
    else:  # duplicate values across bins and generations, a quiescent type, a zero-ratio type
        bins = [(64.0, 30), (32.0, 20), (16.0, 10), (48.0, 7), (3.0, 0), (24.0, 9)]
        types = [(0.5, 9.0, 3.0), (0.0, 12.0, 2.0), (0.5, -1.0, -1.0)]
        t_max, phi, seed = 60.0, 2.0, 77
    p = engine.plan(bins, types, t_max, phi, seed)
    try:
        p.run()
        dev = p.result()
        engine.set_option("device_merge", 0)
        try:
            host = p.result()
        finally:
            engine.set_option("device_merge", 1)
    finally:
        p.close()
    o = oracle_lib.simulate(bins, types, t_max, phi, seed=seed, nthreads=0)
    for r in (dev, host):
        assert np.array_equal(r.values, o.values)
        assert np.array_equal(r.totals, o.totals)
        assert np.array_equal(r.per_type, o.per_type)
    assert dev.stats["leaves"] == host.stats["leaves"] == o.stats["leaves"]


def test_repeat_runs_identical(engine):
    w = cfg.small()
    p = engine.plan(w.bins, w.types, w.t_max, w.phi, w.seed)
    p.run()
    a = p.result()
    p.run()
    b = p.result()
    p.close()
    assert np.array_equal(a.per_type, b.per_type)


def test_invalid_inputs_report_errors(engine):
    from procell import ProcellError
    with pytest.raises(ProcellError, match="PC_ERR_INVALID"):
        engine.simulate([(4.0, 1)], [(0.5, 1.0, 0.1), (0.4, 2.0, 0.1)], 1.0, 1.0)
    with pytest.raises(ProcellError, match="PC_ERR_INVALID"):
        engine.simulate([(4.0, 1)], [(1.0, 1.0, 0.1)], -1.0, 1.0)
    with pytest.raises(ProcellError, match="PC_ERR_INVALID"):
        engine.simulate([(4.0, 1)], [(1.0, 1.0, 0.1)], 1.0, -2.0)
    with pytest.raises(ProcellError, match="PC_ERR_UNSUPPORTED"):
        engine.simulate([(4.0, 1)], [(1.0 / 65, 1.0, 0.1)] * 65, 1.0, 1.0)
    # the context stays usable after errors
    w = cfg.small()
    engine.simulate(w.bins, w.types, w.t_max, w.phi, w.seed)
