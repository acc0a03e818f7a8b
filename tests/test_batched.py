"""The batched form (pc_batch_*): many independent instances in one run.

Every instance of a batch must give the same uint64 counts, bit for bit, as the plain form
(pc_plan_run) on that instance alone with the same seed, and through that the oracle's.
Batches mix uneven instances (different histograms, type sets, t_max, phi, seeds), the
reference's edge cases per instance, and launch geometries whose root chunks and sweep
slices straddle instance boundaries.
"""
import numpy as np
import pytest

import procell.configs as cfg
from procell import ProcellError

pytestmark = pytest.mark.gpu


def inst(w):
    return (w.bins, w.types, w.t_max, w.phi, w.seed)


def plain_counts(engine, bins, types, t_max, phi, seed):
    p = engine.plan(bins, types, t_max, phi, seed)
    try:
        p.run()
        return p.raw_counts(), p.result()
    finally:
        p.close()


def check_batch(engine, instances):
    b = engine.batch(instances)
    try:
        b.run()
        st = b.stats()
        total_roots = 0
        for i, x in enumerate(instances):
            want, want_res = plain_counts(engine, *x)
            got = b.raw_counts(i)
            assert got.shape == want.shape, (i, got.shape, want.shape)
            assert np.array_equal(got, want), (i, np.argwhere(got != want)[:5])
            r = b.result(i)
            assert np.array_equal(r.values, want_res.values)
            assert np.array_equal(r.totals, want_res.totals)
            assert np.array_equal(r.per_type, want_res.per_type)
            assert r.stats["leaves"] == want_res.stats["leaves"]
            assert r.stats["roots"] == want_res.stats["roots"]
            total_roots += want_res.stats["roots"]
        assert st["roots"] == total_roots
        return b, st
    finally:
        b.close()


def small_uneven(n, seed):
    """Instances with the batched generator's shape, sized down so the plain loop is quick."""
    rng = np.random.default_rng(seed)
    ws = cfg.batched(n_instances=n, seed=seed)
    out = []
    for w in ws:
        # keep the histogram, types, t_max and phi; thin the frequencies to <= ~20k cells
        total = sum(f for _, f in w.bins)
        keep = min(1.0, 20_000 / max(1, total)) * rng.uniform(0.2, 1.0)
        bins = [(v, int(f * keep)) for v, f in w.bins]
        nz = [v for v, f in bins if f > 0]
        out.append((bins, w.types, w.t_max, min(nz) if nz else 1.0, w.seed))
    return out


EDGE = [
    # quiescent-only and zero-mean types
    ([(100.0, 50), (3.0, 20)], [(1.0, -1.0, -1.0)], 50.0, 1.0, 5),
    ([(64.0, 300), (7.0, 9)], [(0.6, 0.0, 2.0), (0.4, 5.0, 1.0)], 30.0, 1.0, 6),
    # t_max = 0, phi above every value, zero-frequency rows, an empty histogram
    ([(500.0, 100)], [(1.0, 10.0, 3.0)], 0.0, 1.0, 7),
    ([(5.0, 40), (9.0, 0), (3.0, 12)], [(0.5, 8.0, 2.0), (0.5, 12.0, 6.0)], 100.0, 50.0, 8),
    ([(9.0, 0)], [(1.0, 10.0, 3.0)], 100.0, 1.0, 9),
    # negative-sd and sd > mean (truncation), many types, automatic phi
    ([(2000.0, 500), (37.5, 80)], [(0.5, 10.0, -4.0), (0.5, 3.0, 9.0)], 120.0, None, 10),
    ([(1e4, 200)], [(1.0 / 64, 20.0 + i, 5.0 + 0.1 * i) for i in range(64)], 200.0, 2.0, 11),
]


def test_batch_uneven_matches_plain(engine):
    check_batch(engine, small_uneven(48, seed=21))


def test_batch_edge_instances_match_plain(engine):
    check_batch(engine, EDGE + small_uneven(6, seed=22))


def test_batch_small_config_matches_oracle(engine, oracle_lib):
    w = cfg.small()
    other = cfg.small(seed=3)
    b = engine.batch([inst(other), inst(w), inst(other)])
    try:
        b.run()
        r = b.result(1)
        o = oracle_lib.simulate(w.bins, w.types, w.t_max, w.phi, seed=w.seed, nthreads=0)
        assert np.array_equal(r.values, o.values)
        assert np.array_equal(r.totals, o.totals)
        assert np.array_equal(r.per_type, o.per_type)
        assert np.array_equal(b.raw_counts(0), b.raw_counts(2))
    finally:
        b.close()


def test_batch_wide_key_layout(engine):
    # an instance whose phi cap exceeds 32 generations puts the whole batch on the wide key layout
    deep = ([(2.0 ** 40, 3)], [(1.0, 1.0, 0.05)], 6.0, 1.0, 31)
    check_batch(engine, [deep] + small_uneven(4, seed=23))


@pytest.mark.parametrize("opts", [{"max_root_chunk": 777}, {"max_slice_cells": 5000},
                                  {"grid_blocks": 3}])
def test_batch_geometry_independent(engine, opts):
    instances = small_uneven(12, seed=24)
    ref = engine.batch(instances)
    ref.run()
    want = [ref.raw_counts(i) for i in range(len(instances))]
    ref.close()
    for k, v in opts.items():
        engine.set_option(k, v)
    try:
        b = engine.batch(instances)
        b.run()
        for i in range(len(instances)):
            assert np.array_equal(b.raw_counts(i), want[i]), i
        b.close()
    finally:
        for k in opts:
            engine.set_option(k, 0)


def test_batch_rerun_and_invalid_instance(engine):
    instances = small_uneven(5, seed=25)
    b = engine.batch(instances)
    b.run()
    first = [b.raw_counts(i) for i in range(5)]
    b.run()
    for i in range(5):
        assert np.array_equal(b.raw_counts(i), first[i])
    with pytest.raises(ProcellError, match="instance index out of range"):
        b.result(5)
    b.close()
    bad = list(instances)
    bad[3] = (bad[3][0], [(0.5, 10.0, 1.0)], 10.0, None, 1)
    with pytest.raises(ProcellError, match="instance 3: ERROR: proportion"):
        engine.batch(bad)


def test_batch_of_many_tiny_instances(engine):
    # a thousand instances of a few cells each: bin/class/type tables with many boundaries
    rng = np.random.default_rng(41)
    instances = []
    for i in range(1000):
        nb = int(rng.integers(1, 6))
        bins = [(float(np.exp(rng.uniform(0.0, 7.0))), int(rng.integers(0, 4))) for _ in range(nb)]
        nt = int(rng.integers(1, 4))
        r = rng.dirichlet(np.ones(nt))
        r = r / r.sum()
        types = [(float(r[k]), float(rng.uniform(5.0, 60.0)), float(rng.uniform(0.5, 10.0))) for k in range(nt)]
        if rng.random() < 0.1:
            types[-1] = (types[-1][0], -1.0, -1.0)
        phi = None if any(f for _, f in bins) else 1.0  # automatic phi needs a nonzero row
        instances.append((bins, types, float(rng.uniform(0.0, 150.0)), phi, int(rng.integers(0, 2 ** 40))))
    b = engine.batch(instances)
    b.run()
    for i, x in enumerate(instances):
        want, _ = plain_counts(engine, *x)
        assert np.array_equal(b.raw_counts(i), want), i
    b.close()


def tiny_instances(n, seed):
    rng = np.random.default_rng(seed)
    instances = []
    for i in range(n):
        nb = int(rng.integers(1, 6))
        bins = [(float(np.exp(rng.uniform(0.0, 7.0))), int(rng.integers(0, 40))) for _ in range(nb)]
        nt = int(rng.integers(1, 4))
        r = rng.dirichlet(np.ones(nt))
        types = [(float(r[k]), float(rng.uniform(5.0, 60.0)), float(rng.uniform(0.5, 10.0))) for k in range(nt)]
        phi = None if any(f for _, f in bins) else 1.0
        instances.append((bins, types, float(rng.uniform(0.0, 150.0)), phi, int(rng.integers(0, 2 ** 40))))
    return instances


@pytest.mark.parametrize("n,parts", [(7, 4), (2100, 4), (2100, 3), (2100, 64), (2100, 1)])
def test_simulate_batch_matches_one_batch(engine, n, parts):
    """pc_simulate_batch (host inputs in, merged histograms out) equals pc_batch_result of one
    batch run, instance by instance. It runs n instances as min(batch_parts, n / 256)
    sub-batches (weights 1, 4, ..., 4, 1), preparing the next and merging the previous on host
    threads while the device runs one: results must not change with the split."""
    instances = small_uneven(n, seed=5) if n < 100 else tiny_instances(n, seed=77)
    engine.set_option("batch_parts", parts)
    try:
        got = engine.simulate_batch(instances)
    finally:
        engine.set_option("batch_parts", 4)
    b = engine.batch(instances)
    try:
        b.run()
        for i in range(n):
            want = b.result(i)
            assert np.array_equal(got[i].values, want.values), i
            assert np.array_equal(got[i].totals, want.totals), i
            assert np.array_equal(got[i].per_type, want.per_type), i
            assert got[i].stats["leaves"] == want.stats["leaves"], i
            assert got[i].stats["roots"] == want.stats["roots"], i
    finally:
        b.close()


def test_batch_parts_option_bounds(engine):
    """batch_parts takes 1..64; other values are rejected."""
    for bad in (0, 65, 0.5):
        with pytest.raises(ProcellError):
            engine.set_option("batch_parts", bad)
    engine.set_option("batch_parts", 64)
    engine.set_option("batch_parts", 4)


def test_set_types_and_totals(engine):
    """pc_batch_set_types re-parameterises a prepared batch: the next run equals a batch
    created with the new types, instance by instance; pc_batch_totals returns every
    instance's merged totals at once; invalid types leave the batch unchanged."""
    import procell.configs as cfg
    ws = cfg.batched(n_instances=12, seed=5)
    ws = [w for w in ws if w.roots <= 200_000][:6]
    inst = [(w.bins, w.types, w.t_max, w.phi, w.seed) for w in ws]
    rng = np.random.default_rng(3)
    new_types = []
    for w in ws:
        k = len(w.types)
        r = rng.dirichlet(np.ones(k))
        new_types.append([(float(r[j]), float(rng.uniform(25, 90)) if w.types[j][1] >= 0 else -1.0,
                           float(rng.uniform(3, 20)) if w.types[j][1] >= 0 else -1.0) for j in range(k)])
    b = engine.batch(inst)
    b.run()
    before = [b.result(i).totals for i in range(len(ws))]
    flat = [t for ts in new_types for t in ts]
    b.set_types(flat)
    with pytest.raises(Exception):
        b.result(0)  # the previous counts belong to the previous types
    b.run()
    off, tot = b.totals()
    ref = engine.batch([(w.bins, new_types[i], w.t_max, w.phi, w.seed) for i, w in enumerate(ws)])
    ref.run()
    for i in range(len(ws)):
        r = ref.result(i)
        assert np.array_equal(b.result(i).per_type, r.per_type), i
        assert np.array_equal(tot[off[i]:off[i + 1]], r.totals), i
    ref.close()
    bad = list(flat)
    bad[0] = (bad[0][0] + 0.5, bad[0][1], bad[0][2])  # ratios no longer sum to 1
    with pytest.raises(Exception, match="instance 0"):
        b.set_types(bad)
    b.run()
    assert np.array_equal(b.totals()[1], tot)
    b.set_types([t for w in ws for t in w.types])
    b.run()
    for i in range(len(ws)):
        assert np.array_equal(b.result(i).totals, before[i]), i
    b.close()
