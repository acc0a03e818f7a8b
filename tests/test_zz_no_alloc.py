"""The allocation-free entry point, pc_simulate_noalloc, against the regular one.

pc_simulate_noalloc serves callers that may not allocate device memory (a host application
whose own pool owns the GPU, code that must not trigger cudaMalloc's implicit
synchronisation, deployments with a fixed memory budget): everything lives in one static
device array shared by all calls. These checks call it through the C ABI twice in a row
(the second call sees the first call's leftovers in that array) and require the same
uint64 counts, bit for bit, as pc_plan_run + pc_plan_raw_counts on the same inputs and seed.
The inputs include one of about 1e6 initial cells, larger than one root chunk of the fixed
array (so several chunks run and levels are cut into slices), one whose cell types are
listed in ascending ratio order (the counts must come back in file order), and one whose
lineages are deeper than 32 generations (the wide key layout); those three are also merged
into the output value set and compared with the oracle directly.

Out-of-memory rejection is tested on an input whose tables alone exceed the array. The
other rejection, a lineage deeper than the array's level buffers, needs more than 40
generations of divisions in one lineage, i.e. on the order of 2^40 cells, and is left out.

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


def merged_from_raw(raw, bins, phi):
    """The output value set's counts from raw [generation][bin][type] counts: a leaf of
    generation g in bin b has the value v_b / 2^g (src/io/parser.cu:126-137)."""
    vals = np.array([v for v, f in bins if f], np.float64)
    out = {}
    for g in range(raw.shape[0]):
        for b in np.flatnonzero(raw[g].sum(axis=1)):
            v = float(np.ldexp(vals[b], -g))
            out[v] = out.get(v, 0) + raw[g, b].astype(np.uint64)
    return out


def assert_matches_oracle(oracle_lib, raw, bins, types, t_max, phi, seed):
    o = oracle_lib.simulate(bins, types, t_max, phi, seed=seed, nthreads=0)
    got = merged_from_raw(raw, bins, phi)
    nz = np.flatnonzero(o.totals)
    assert sorted(got) == [float(v) for v in o.values[nz]]
    for i in nz:
        assert np.array_equal(got[float(o.values[i])], o.per_type[i]), o.values[i]
    return o


MEDIUM = cfg.medium()
CASES = {
    "small": (lambda w: (w.bins, w.types, w.t_max, w.phi, w.seed))(cfg.small()),
    "edge": ([(1000.0, 7), (3.0, 0), (0.5, 9), (64.0, 300)],
             [(0.5, 6.0, 2.0), (0.3, 0.0, 1.0), (0.2, -1.0, -1.0)], 40.0, 1.0, 99),
    # about 1e6 initial cells: several root chunks of the fixed array, sliced levels
    "medium": (MEDIUM.bins, MEDIUM.types, MEDIUM.t_max, MEDIUM.phi, MEDIUM.seed),
    # the same with the types listed in ascending ratio order (sorted order != file order)
    "medium_types_ascending": (MEDIUM.bins, MEDIUM.types[::-1], MEDIUM.t_max, MEDIUM.phi, MEDIUM.seed + 1),
    # phi cap above 32 generations: the wide key layout
    "wide_keys": ([(2.0 ** 40, 5), (2.0 ** 36, 3), (5.0, 4)], [(0.6, 10.0, 2.0), (0.4, 12.0, 3.0)],
                  200.0, 1.0, 7),
    # phi cap exactly 32 with lineages through generation 31: parked generation-32 daughters
    # carry keys one generation deeper than any stored cell
    "narrow_boundary": ([(2.0 ** 32.5, 3)], [(1.0, 1.0, 0.5)], 22.0, 1.0, 12345),
}
ORACLE_CASES = ("medium", "medium_types_ascending", "wide_keys", "narrow_boundary")


@pytest.mark.parametrize("name", sorted(CASES))
def test_noalloc_matches_regular_twice(engine, oracle_lib, name):
    bins, types, t_max, phi, seed = CASES[name]
    want, want_stats = regular_counts(engine, bins, types, t_max, phi, seed)
    for _ in range(2):
        rc, out, dims, st, err = noalloc_counts(bins, types, t_max, phi, seed, want.size)
        assert rc == 0, err
        assert dims == want.shape
        assert np.array_equal(out[:want.size].reshape(want.shape), want)
        assert st.divisions == want_stats["divisions"] and st.vanished == want_stats["vanished"]
        assert st.uncounted == want_stats["uncounted"]
    if name in ORACLE_CASES:
        o = assert_matches_oracle(oracle_lib, out[:want.size].reshape(want.shape), bins, types, t_max, phi, seed)
        assert st.divisions == o.stats["divisions"] and st.vanished == o.stats["vanished"]
    if name == "medium":
        assert st.root_sweeps >= 3 and st.divisions > st.root_sweeps * 100_000  # several chunks and slices
    if name == "wide_keys":
        assert dims[0] > 34 and st.max_generation > 0


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
