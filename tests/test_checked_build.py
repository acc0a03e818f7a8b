"""The checked build: the kernels compiled with PC_CHECKED, which guards every level-segment
write and read, root-record access and count-table update with a bounds check that sets
error bit 16 (and skips the access) instead of trapping. It stands in for a memory sanitizer,
which this machine's GPUs do not offer; the reference has neither (its level buffers are
read uninitialised, src/simulation/proliferation.cu:230-238, :315).

The small and medium workloads run on the checked library in both drivers and through the
allocation-free entry point; every run must finish with no check failed and counts
bit-identical to the oracle's.
"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cuda-pro-cell_gb300")

SCRIPT = r'''
import ctypes, sys
import numpy as np
import oracle
import procell.configs as cfg
from procell import Engine, _lib
assert _lib.LIB_PATH.endswith("build_checked/libprocell.so"), _lib.LIB_PATH
eng = Engine(0)
for name in ("small", "medium"):
    w = cfg.by_name(name)
    o = oracle.simulate(w.bins, w.types, w.t_max, w.phi, seed=w.seed, nthreads=0)
    for driver, graph in ((0, 0), (1, 0), (1, 1)):
        eng.set_option("driver", driver)
        eng.set_option("graph", graph)
        g = eng.simulate(w.bins, w.types, w.t_max, w.phi, w.seed)  # raises on a failed check
        assert np.array_equal(g.per_type, o.per_type), (name, driver, graph)
        assert g.stats["divisions"] == o.stats["divisions"]
    # the batched form: the workload and a variant with its types reversed, in one batch
    b = eng.batch([(w.bins, w.types, w.t_max, w.phi, w.seed), (w.bins, w.types[::-1], w.t_max, w.phi, w.seed)])
    b.run()
    assert np.array_equal(b.result(0).per_type, o.per_type), name
    b.close()
# the allocation-free entry point on the small workload
w = cfg.small()
L = _lib.load()
p = eng.plan(w.bins, w.types, w.t_max, w.phi, w.seed)
p.run()
want = p.raw_counts()
p.close()
out = np.zeros(want.size, np.uint64)
dims = (ctypes.c_uint32 * 3)()
st = _lib.Stats()
err = ctypes.create_string_buffer(256)
rc = L.pc_simulate_noalloc(_lib.bins_array(w.bins), len(w.bins), _lib.types_array(w.types), len(w.types),
                           float(w.t_max), float(w.phi), int(w.seed), None,
                           out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), want.size, dims,
                           ctypes.byref(st), err, len(err))
assert rc == 0, err.value
assert np.array_equal(out.reshape(want.shape), want)
eng.close()
print("checked build ok")
'''


def test_checked_build_runs_clean_on_small_and_medium(built, oracle_lib):
    lib = built.build(out=os.path.join(PKG, "build_checked"), defines=["PC_CHECKED=1"])
    env = dict(os.environ, PROCELL_LIB=lib,
               PYTHONPATH=os.pathsep.join([PKG, os.path.join(ROOT, "oracle"), os.environ.get("PYTHONPATH", "")]))
    r = subprocess.run([sys.executable, "-c", SCRIPT], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-3000:])
    assert "checked build ok" in r.stdout
