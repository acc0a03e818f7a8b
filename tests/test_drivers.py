"""Every compiled sweep configuration and both drivers give the same counts, bit for bit.

The configurations (threads per block x cells per lane x leaf-count privatisation) and the
drivers (one launch per sweep; one persistent cooperative launch, optionally replayed from
a captured CUDA graph) change only how the work is scheduled, never a random draw or a
rounding, so every combination must reproduce the oracle's histogram exactly.
"""
import itertools

import numpy as np
import pytest

import procell.configs as cfg

pytestmark = pytest.mark.gpu

CONFIGS = list(range(8))
DRIVERS = [(0, 0), (1, 0), (1, 1)]  # (driver, graph)


def set_opts(engine, **opts):
    for k, v in opts.items():
        engine.set_option(k, v)


def reset(engine):
    set_opts(engine, sweep_config=4, driver=0, graph=0, max_slice_cells=0, max_root_chunk=0, grid_blocks=0)


@pytest.fixture
def eng(engine):
    reset(engine)
    yield engine
    reset(engine)


@pytest.fixture(scope="module")
def small_oracle(oracle_lib):
    w = cfg.small()
    return w, oracle_lib.simulate(w.bins, w.types, w.t_max, w.phi, seed=w.seed, nthreads=0)


@pytest.mark.parametrize("config,driver", list(itertools.product(CONFIGS, DRIVERS)))
def test_small_every_config_and_driver(eng, small_oracle, config, driver):
    w, o = small_oracle
    set_opts(eng, sweep_config=config, driver=driver[0], graph=driver[1])
    g = eng.simulate(w.bins, w.types, w.t_max, w.phi, w.seed)
    assert np.array_equal(g.totals, o.totals)
    assert np.array_equal(g.per_type, o.per_type)
    for k in ("divisions", "leaves", "uncounted", "vanished"):
        assert g.stats[k] == o.stats[k], k
    assert g.stats["max_generation"] == o.stats["max_gen"]


@pytest.mark.parametrize("driver", DRIVERS)
def test_medium_persistent_matches_per_sweep(eng, driver):
    w = cfg.medium()
    p = eng.plan(w.bins, w.types, w.t_max, w.phi, w.seed)
    p.run()
    want, want_st = p.raw_counts(), p.stats()
    set_opts(eng, sweep_config=7, driver=driver[0], graph=driver[1])
    for _ in range(2):  # the second run replays the captured graph
        p.run()
        assert np.array_equal(p.raw_counts(), want)
        st = p.stats()
        for k in ("divisions", "vanished", "uncounted", "max_generation"):
            assert st[k] == want_st[k], k
    p.close()


@pytest.mark.parametrize("opts", [{"max_slice_cells": 3000}, {"max_root_chunk": 1000},
                                  {"grid_blocks": 5}, {"max_slice_cells": 700, "max_root_chunk": 333}])
def test_persistent_many_sweeps_and_chunks(eng, small_oracle, opts):
    w, o = small_oracle
    set_opts(eng, driver=1, graph=1, **opts)
    g = eng.simulate(w.bins, w.types, w.t_max, w.phi, w.seed)
    assert np.array_equal(g.per_type, o.per_type)
    assert g.stats["divisions"] == o.stats["divisions"]


def test_graph_recaptured_when_roots_change(eng, oracle_lib):
    w = cfg.small()
    set_opts(eng, driver=1, graph=1)
    p = eng.plan(w.bins, w.types, w.t_max, w.phi, w.seed)
    n = w.roots
    for lo, hi in [(0, n), (n // 3, n), (0, n // 2), (0, n)]:
        p.set_roots(lo, hi)
        p.run()
        r = p.result()
        o = oracle_lib.simulate(w.bins, w.types, w.t_max, w.phi, seed=w.seed, root_begin=lo, root_end=hi,
                                nthreads=0)
        assert np.array_equal(r.per_type, o.per_type), (lo, hi)
    p.close()


def test_persistent_wide_layout(eng, oracle_lib):
    bins = [(2.0 ** 40, 5), (3000.0, 40)]
    types = [(0.7, 1.0, 0.05), (0.3, 2.0, 0.5)]
    o = oracle_lib.simulate(bins, types, 7.0, 1.0, seed=3, nthreads=0)
    for drv, graph in DRIVERS:
        set_opts(eng, driver=drv, graph=graph)
        g = eng.simulate(bins, types, 7.0, 1.0, 3)
        assert np.array_equal(g.per_type, o.per_type)


@pytest.mark.parametrize("config", [0, 3, 4, 7])
def test_batched_persistent_every_config(eng, config):
    from test_batched import small_uneven
    instances = small_uneven(10, seed=31)
    b = eng.batch(instances)
    b.run()
    want = [b.raw_counts(i) for i in range(len(instances))]
    set_opts(eng, sweep_config=config, driver=1, graph=1)
    for _ in range(2):
        b.run()
        for i in range(len(instances)):
            assert np.array_equal(b.raw_counts(i), want[i]), i
    b.close()


def test_autotune_picks_a_compiled_combination(eng, small_oracle):
    w, o = small_oracle
    p = eng.plan(w.bins, w.types, w.t_max, w.phi, w.seed)
    t = eng.autotune(p, repeats=1)
    assert t["candidates"] == 16 and 0 <= t["config"] < 8 and t["driver"] in (0, 1)
    assert t["threads"] in (128, 256) and t["cells_per_lane"] in (1, 2)
    assert 0 < t["ms"] <= t["ms_default"]
    p.run()
    r = p.result()
    assert np.array_equal(r.per_type, o.per_type)
    p.close()


def test_barrier_timeout_is_reported_and_the_context_survives(eng, small_oracle):
    """Failure detection of the persistent driver without a GPU fault: a grid barrier that
    can never complete (its arrival counter preset) runs into its time limit, every block
    returns with error bit 2 set, and the context keeps working."""
    import ctypes
    L = eng.L
    err, passed = ctypes.c_uint32(), ctypes.c_uint32()
    assert L.pc_debug_barrier(eng.ctx, 0, 100.0, ctypes.byref(err), ctypes.byref(passed)) == 0
    assert err.value == 0 and passed.value >= 1
    blocks = passed.value
    assert L.pc_debug_barrier(eng.ctx, 1, 100.0, ctypes.byref(err), ctypes.byref(passed)) == 0
    assert err.value & 4 and passed.value == 0
    assert L.pc_debug_barrier(eng.ctx, 0, 100.0, ctypes.byref(err), ctypes.byref(passed)) == 0
    assert err.value == 0 and passed.value == blocks
    w, o = small_oracle
    set_opts(eng, driver=1, graph=1)
    g = eng.simulate(w.bins, w.types, w.t_max, w.phi, w.seed)
    assert np.array_equal(g.per_type, o.per_type)


def test_barrier_timeout_reaches_blocks_waiting_elsewhere(eng, small_oracle):
    """Every block leaves within one poll period of the first timeout: in a second barrier
    that can never complete (one block skips it), one block waits with a 100 ms limit and the
    others with 10 s; the call returns long before 10 s only because the waiting blocks poll
    the error bit that the first block's timeout sets. The context keeps working."""
    import ctypes
    import time
    L = eng.L
    err, passed = ctypes.c_uint32(), ctypes.c_uint32()
    t0 = time.perf_counter()
    assert L.pc_debug_barrier(eng.ctx, 2, 100.0, ctypes.byref(err), ctypes.byref(passed)) == 0
    dt = time.perf_counter() - t0
    assert err.value & 4 and passed.value == 0
    assert dt < 2.0, dt
    w, o = small_oracle
    set_opts(eng, driver=1, graph=0)
    g = eng.simulate(w.bins, w.types, w.t_max, w.phi, w.seed)
    assert np.array_equal(g.per_type, o.per_type)
