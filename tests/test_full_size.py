"""Full-size checks through properties that do not depend on size.

The oracle finishes the small and medium workloads and 1/200 of the large one (the bit-exact
tests); at the large workload's full size (1e7 initial cells, 3.6e9 divisions) and the
batched workload's (6e8 initial cells) the engine is checked through properties that hold
for any size: conservation of cells, additivity over shards of the initial cells, identical
counts under every driver and compiled configuration, and, for the batched form, per
instance equality with the plain form.
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
