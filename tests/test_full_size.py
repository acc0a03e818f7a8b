"""Full-size checks: bit-exact against the oracle, and properties that do not depend on size.

The large workload (4096 bins, 1e7 initial cells, 3.6e9 divisions) is compared in full with
the oracle run on every host core (about 20 s on 16 cores), as are 64 instances of the
4096-instance batched workload, drawn at random, at their full size. Beside that, the
engine is checked through properties that hold for any size: conservation of cells,
additivity over shards of the initial cells, identical counts under every driver and
compiled configuration, and, for the batched form, per instance equality with the plain
form.
"""
import numpy as np
import pytest

import procell.configs as cfg

pytestmark = pytest.mark.gpu


def set_opts(engine, **opts):
    for k, v in opts.items():
        engine.set_option(k, v)


@pytest.fixture(scope="module")
def large_full(engine):
    w = cfg.large()
    set_opts(engine, sweep_config=4, driver=0, graph=0)
    p = engine.plan(w.bins, w.types, w.t_max, w.phi, w.seed)
    p.run()
    raw, res, st = p.raw_counts(), p.result(), p.stats()
    yield w, p, raw, res, st
    p.close()


def test_large_conservation(large_full):
    w, _, raw, res, st = large_full
    # every initial cell and every division's second daughter ends as exactly one of: a
    # counted leaf, an uncounted generation-0 leaf (value below phi), a vanished cell
    assert st["roots"] == w.roots
    assert st["roots"] + st["divisions"] == res.stats["leaves"] + st["uncounted"] + st["vanished"]
    assert int(raw.sum()) == res.stats["leaves"] == int(res.totals.sum())
    assert st["divisions"] > 3_000_000_000
    v = res.values
    assert np.all(np.diff(v) > 0) and v[0] >= w.phi


def assert_same(g, o):
    assert np.array_equal(g.values, o.values)
    assert np.array_equal(g.totals, o.totals), np.flatnonzero(g.totals != o.totals)[:10]
    assert np.array_equal(g.per_type, o.per_type)
    for k in ("roots", "divisions", "leaves", "uncounted", "vanished"):
        assert g.stats[k] == o.stats[k], (k, g.stats[k], o.stats[k])
    assert g.stats["max_generation"] == o.stats["max_gen"]


def test_large_full_size_bit_exact_vs_oracle(oracle_lib, large_full):
    # every one of the 1e7 initial cells: the same chunking, slicing and leaf counts as
    # the benchmarked run, against the CPU restatement of proliferation.cu:289-410
    w, _, _, res, _ = large_full
    o = oracle_lib.simulate(w.bins, w.types, w.t_max, w.phi, seed=w.seed, nthreads=0)
    assert o.stats["divisions"] > 3_000_000_000
    assert_same(res, o)


def test_batched_workload_instances_bit_exact_vs_oracle(engine, oracle_lib):
    # the benchmark's 4096-instance batch in one run; 64 instances drawn at random are
    # each compared in full with the oracle's run of that instance alone
    ws = cfg.batched()
    b = engine.batch([(w.bins, w.types, w.t_max, w.phi, w.seed) for w in ws])
    try:
        b.run()
        pick = np.random.default_rng(2024).choice(len(ws), size=64, replace=False)
        for i in sorted(int(x) for x in pick):
            w = ws[i]
            o = oracle_lib.simulate(w.bins, w.types, w.t_max, w.phi, seed=w.seed, nthreads=0)
            g = b.result(i)
            assert np.array_equal(g.values, o.values), i
            assert np.array_equal(g.per_type, o.per_type), i
            assert np.array_equal(g.totals, o.totals), i
    finally:
        b.close()


def test_large_shards_add_up(engine, large_full):
    w, p, raw, _, st = large_full
    n = w.roots
    cuts = [0, n // 3, (2 * n) // 3, n]
    total = np.zeros_like(raw)
    divisions = 0
    for a, b in zip(cuts, cuts[1:]):
        p.set_roots(a, b)
        p.run()
        total += p.raw_counts()
        divisions += p.stats()["divisions"]
    p.set_roots(0, n)
    assert np.array_equal(total, raw)
    assert divisions == st["divisions"]


@pytest.mark.parametrize("opts", [{"driver": 1, "graph": 1}, {"sweep_config": 7}, {"sweep_config": 0, "driver": 1}])
def test_large_every_driver_identical(engine, large_full, opts):
    _, p, raw, _, st = large_full
    try:
        set_opts(engine, **opts)
        p.run()
        assert np.array_equal(p.raw_counts(), raw)
        assert p.stats()["divisions"] == st["divisions"]
    finally:
        set_opts(engine, sweep_config=4, driver=0, graph=0)


def test_batched_full_size_instances_match_plain(engine):
    # 256 instances of the batched workload at their full size (up to 1e6 cells each)
    ws = cfg.batched(n_instances=256, seed=77)
    instances = [(w.bins, w.types, w.t_max, w.phi, w.seed) for w in ws]
    b = engine.batch(instances)
    b.run()
    st = b.stats()
    assert st["roots"] == sum(w.roots for w in ws)
    for i, x in enumerate(instances):
        p = engine.plan(*x)
        p.run()
        assert np.array_equal(b.raw_counts(i), p.raw_counts()), i
        p.close()
    b.close()
