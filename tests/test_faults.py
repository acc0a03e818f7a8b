"""Failure detection by host-side fault injection (no GPU fault is ever provoked).

The reference checks no CUDA status at all (src/simulation/proliferation.cu:26-284). Here
every CUDA call the library makes is checked and returned as a status. With the option
fail_nth_call = n, the n-th call from then on (allocation, copy, memset, synchronisation,
event record, kernel or graph launch) does not reach CUDA and fails once instead. For every
n over all the calls of a run, in each driver and in the batched and smoothed forms, the
checks require: the failure comes back as PC_ERR_NOMEM or PC_ERR_CUDA (or the library
recovers from it and the result is still exact), exactly one fault was injected, the next
call on the same context is bit-exact against the oracle, and the library's live device
allocations and level buffers are what a clean run leaves (nothing leaked).
"""
import numpy as np
import pytest

import procell.configs as cfg
from procell import ProcellError

pytestmark = pytest.mark.gpu

PC_ERR_CUDA, PC_ERR_NOMEM = 2, 3


@pytest.fixture(scope="module")
def small_oracle(oracle_lib):
    w = cfg.small()
    return w, oracle_lib.simulate(w.bins, w.types, w.t_max, w.phi, seed=w.seed, nthreads=0)


def counters(eng):
    return eng.get_option("device_allocations"), eng.get_option("level_buffers")


def sweep_faults(eng, run, check):
    """Inject a failure at every CUDA call of `run()` in turn; `check(result)` validates a
    successful result. Returns the number of calls covered."""
    check(run())  # warm: pool, spare buffers and graphs in their steady state
    c0 = eng.get_option("cuda_calls")
    check(run())
    ncalls = int(eng.get_option("cuda_calls") - c0)
    assert ncalls > 0
    clean = counters(eng)
    for n in range(1, ncalls + 1):
        f0 = eng.get_option("faults_injected")
        eng.set_option("fail_nth_call", n)
        try:
            check(run())  # the library recovered (e.g. a graph that could not be captured)
        except ProcellError as e:
            assert e.code in (PC_ERR_CUDA, PC_ERR_NOMEM), (n, e)
        eng.set_option("fail_nth_call", 0)
        assert eng.get_option("faults_injected") == f0 + 1, n
        check(run())
        assert counters(eng) == clean, (n, counters(eng), clean)
    return ncalls


@pytest.mark.parametrize("driver,graph", [(0, 0), (1, 0), (1, 1)])
def test_every_failing_call_of_a_run_is_reported(engine, small_oracle, driver, graph):
    w, o = small_oracle
    engine.set_option("driver", driver)
    engine.set_option("graph", graph)
    try:
        def run():
            return engine.simulate(w.bins, w.types, w.t_max, w.phi, w.seed)

        def check(g):
            assert np.array_equal(g.per_type, o.per_type) and g.stats["divisions"] == o.stats["divisions"]

        assert sweep_faults(engine, run, check) >= 8
    finally:
        engine.set_option("driver", 0)
        engine.set_option("graph", 0)


def test_every_failing_call_of_a_batch_is_reported(engine, oracle_lib, small_oracle):
    w, o = small_oracle
    o2 = oracle_lib.simulate(w.bins, w.types[::-1], w.t_max, w.phi, seed=w.seed + 1, nthreads=0)
    instances = [(w.bins, w.types, w.t_max, w.phi, w.seed), (w.bins, w.types[::-1], w.t_max, w.phi, w.seed + 1)]

    def run():
        b = engine.batch(instances)
        try:
            b.run()
            return b.result(0), b.result(1)
        finally:
            b.close()

    def check(r):
        assert np.array_equal(r[0].per_type, o.per_type) and np.array_equal(r[1].per_type, o2.per_type)

    assert sweep_faults(engine, run, check) >= 8


def test_every_failing_call_of_the_smoothed_form_is_reported(engine):
    import torch
    from procell.smooth import Smooth
    bins = [(640.0, 30), (37.0, 20), (3.0, 10)]
    P = torch.tensor([[[0.6, 30.0, 6.0], [0.4, 45.0, 9.0]]], dtype=torch.float64, device="cuda")
    sm0 = Smooth(engine, bins, n_types=2, t_max=150.0, phi=1.0, h=0.5, paths=2, seed=5)
    E0 = sm0.forward(P).cpu().numpy()
    G0 = sm0.backward(P, torch.ones_like(sm0.forward(P))).cpu().numpy()
    sm0.close()

    def run():
        sm = Smooth(engine, bins, n_types=2, t_max=150.0, phi=1.0, h=0.5, paths=2, seed=5)
        try:
            E = sm.forward(P)
            G = sm.backward(P, torch.ones_like(E))
            sm.sync()
            return E.cpu().numpy(), G.cpu().numpy()
        finally:
            sm.close()

    def check(r):
        assert np.array_equal(r[0], E0) and np.array_equal(r[1], G0)

    assert sweep_faults(engine, run, check) >= 4
