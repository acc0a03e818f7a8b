"""The root chunk and key layout (pc::key_layout in csrc/pc_api.cpp, shared by plans, batches
and the allocation-free path) on the host.

A key names a tree node: narrow layout root_local << 32 | heap node (2^g + path), wide
layout root_local * 2^g + path. Keys exist for the stored cells (generation g <= g_store_max,
g < their phi cap) and for the daughters of the deepest of them, one generation further,
which the division sweep parks with a key when their first draw is not settled. So every
generation up to min(gmax, g_store_max + 1) must fit: root bits + g <= 64 (wide), g <= 31
with root_local < 2^32 (narrow). A layout one bit short put a parked daughter's key into the
root field (a phi cap of exactly 32 in the narrow layout; more than 2^(64 - gmax) roots in
one chunk in the wide one).
"""
import ctypes
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "cuda-pro-cell_gb300", "csrc")


@pytest.fixture(scope="module")
def layout(built, tmp_path_factory):
    from procell import _lib
    out = str(tmp_path_factory.mktemp("layout") / "libkey_layout.so")
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "key_layout.cpp"), "-o", out, "-L" + libdir, "-lprocell",
                    "-Wl,-rpath," + libdir], check=True)
    ctypes.CDLL(_lib.LIB_PATH, mode=ctypes.RTLD_GLOBAL)
    lib = ctypes.CDLL(out)
    lib.layout.restype = None
    lib.layout.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int, ctypes.c_uint64,
                           ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_int)]

    lib.value_set.restype = ctypes.c_int
    lib.value_set.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double, ctypes.c_void_p, ctypes.c_uint64,
                              ctypes.POINTER(ctypes.c_uint64)]

    def call(roots, gmax, batched=False, max_root_chunk=0):
        c, g, n = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_int()
        lib.layout(roots, gmax, int(batched), max_root_chunk, ctypes.byref(c), ctypes.byref(g), ctypes.byref(n))
        return c.value, g.value, bool(n.value)
    call.lib = lib
    return call


def bits_for(n):  # bits needed for values in [0, n)
    return 0 if n <= 1 else (n - 1).bit_length()


ROOTS = sorted({1, 2, 3, 7, 1000, 10_235_694, 2 ** 24 - 1, 2 ** 24, 2 ** 24 + 1, 2 ** 25, 2 ** 28 + 5,
                2 ** 31, 2 ** 32 - 1, 2 ** 32, 2 ** 32 + 1, 2 ** 40, 2 ** 63})


def test_every_key_generation_fits(layout):
    for batched in (False, True):
        for max_chunk in (0, 77_777):
            for roots in ROOTS:
                for gmax in range(0, 70):
                    chunk, gsm, narrow = layout(roots, gmax, batched, max_chunk)
                    where = (roots, gmax, batched, max_chunk, chunk, gsm, narrow)
                    assert 1 <= chunk <= max(1, roots), where
                    assert gsm <= 62, where
                    deepest = min(gmax, gsm + 1)  # stored cells and their parked daughters
                    assert bits_for(chunk) + deepest <= 64, where
                    assert narrow == (gmax <= 31), where
                    if narrow:
                        assert deepest <= 31 and chunk <= 2 ** 32, where
                    if gmax < 45:  # the chunk is cut so that no phi cap needs clamping
                        assert gsm + 1 >= gmax, where


def test_boundary_inputs(layout):
    # a phi cap of exactly 32: the wide layout (keys of generation 32 exist)
    assert layout(3, 32)[2] is False
    assert layout(3, 31)[2] is True
    # gmax 40 with 2^25 roots: the chunk keeps 24 root bits, so generation-40 keys fit
    chunk, gsm, _ = layout(2 ** 25, 40)
    assert bits_for(chunk) + 40 <= 64 and gsm >= 39


def test_value_set_equals_the_oracle(layout, oracle_lib):
    """The output value set (the halving chains v, v/2, ... >= phi of the nonzero bins, sorted
    and deduplicated; parser.cu:98-151) as the engine builds it on the host, against the
    oracle's, on histograms with duplicate values, shared mantissas, automatic phi and a
    wide range of exponents."""
    import numpy as np
    from procell import _lib
    rng = np.random.default_rng(11)
    for trial in range(60):
        nb = int(rng.integers(1, 400))
        kind = trial % 4
        if kind == 0:
            v = np.exp(rng.uniform(0.0, np.log(1e6), nb))
        elif kind == 1:
            v = np.ldexp(1.0 + rng.integers(0, 8, nb) / 8.0, rng.integers(0, 30, nb))
        elif kind == 2:
            v = rng.integers(1, 50, nb).astype(np.float64)
        else:
            v = np.exp(rng.uniform(np.log(1e-30), np.log(1e30), nb))
        f = rng.integers(0, 4, nb)
        bins = list(zip(v.tolist(), f.tolist()))
        phi = [None, 1.0, 1e-6][trial % 3]
        b = _lib.bins_numpy(bins)
        cap = 1 << 20
        out = np.zeros(cap, np.float64)
        n = ctypes.c_uint64()
        rc = layout.lib.value_set(b.ctypes.data, len(b), 0.0 if phi is None else phi, out.ctypes.data, cap,
                                  ctypes.byref(n))
        o = oracle_lib.simulate(bins, [(1.0, 1.0, 0.0)], 0.0, phi, seed=1, nthreads=1)
        if f.sum() == 0:
            continue
        assert rc == 0, (trial, rc)
        assert np.array_equal(out[:n.value], o.values), trial
