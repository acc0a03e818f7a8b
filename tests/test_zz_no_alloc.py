"""The allocation-free entry point, pc_simulate_noalloc, against the regular one.

pc_simulate_noalloc serves callers that may not allocate device memory (a host application
whose own pool owns the GPU, code that must not trigger cudaMalloc's implicit
synchronisation, deployments with a fixed memory budget): everything lives in one static
device array shared by all calls. These checks call it through the C ABI twice in a row
(the second call sees the first call's leftovers in that array) and require the same
uint64 counts, bit for bit, as pc_plan_run + pc_plan_raw_counts on the same inputs and seed.

This file is collected last so that a failure here leaves every other test already run; it
also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import procell.configs as cfg

pytestmark = pytest.mark.gpu


def regular_counts(engine, bins, types, t_max, phi, seed):
    p = engine.plan(bins, types, t_max, phi, seed)
    try:
        p.run()
        return p.raw_counts(), p.stats()
    finally:
        p.close()


def noalloc_counts(bins, types, t_max, phi, seed, capacity):
    from procell import _lib
    L = _lib.load()
    out = np.zeros(max(1, capacity), np.uint64)
    dims = (ctypes.c_uint32 * 3)()
    st = _lib.Stats()
    err = ctypes.create_string_buffer(256)
    rc = L.pc_simulate_noalloc(_lib.bins_array(bins), len(bins), _lib.types_array(types), len(types),
                               float(t_max), 0.0 if phi is None else float(phi), int(seed), None,
                               out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), int(capacity),
                               dims, ctypes.byref(st), err, len(err))
    return rc, out, tuple(dims), st, err.value.decode()


CASES = {
    "small": (lambda w: (w.bins, w.types, w.t_max, w.phi, w.seed))(cfg.small()),
    "edge": ([(1000.0, 7), (3.0, 0), (0.5, 9), (64.0, 300)],
             [(0.5, 6.0, 2.0), (0.3, 0.0, 1.0), (0.2, -1.0, -1.0)], 40.0, 1.0, 99),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_noalloc_matches_regular_twice(engine, name):
    bins, types, t_max, phi, seed = CASES[name]
    want, want_stats = regular_counts(engine, bins, types, t_max, phi, seed)
    for _ in range(2):
        rc, out, dims, st, err = noalloc_counts(bins, types, t_max, phi, seed, want.size)
        assert rc == 0, err
        assert dims == want.shape
        assert np.array_equal(out[:want.size].reshape(want.shape), want)
        assert st.divisions == want_stats["divisions"] and st.vanished == want_stats["vanished"]
        assert st.uncounted == want_stats["uncounted"]


def test_noalloc_reports_sizes(built):
    w = cfg.small()
    rc, _, dims, _, err = noalloc_counts(w.bins, w.types, w.t_max, w.phi, w.seed, 0)
    assert rc == 1 and "raw count buffer" in err
    assert dims[1] == sum(1 for _, f in w.bins if f) and dims[2] == len(w.types) and dims[0] > 1
    # inputs beyond the static array are rejected with a message, not attempted
    # (2M one-cell bins need 88 MB of rows, tables and counts before any level buffer)
    many = [(2.5, 1)] * 2_000_000
    rc, _, _, _, err = noalloc_counts(many, [(1.0, 5.0, 1.0)], 10.0, 1.0, 1, 4_000_000)
    assert rc == 3 and "allocation-free scratch" in err
