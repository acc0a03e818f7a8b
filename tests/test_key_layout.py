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
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", os.path.join(ROOT, "tests", "key_layout.cpp"),
                    "-o", out, "-L" + libdir, "-lprocell", "-Wl,-rpath," + libdir], check=True)
    ctypes.CDLL(_lib.LIB_PATH, mode=ctypes.RTLD_GLOBAL)
    lib = ctypes.CDLL(out)
    lib.layout.restype = None
    lib.layout.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int, ctypes.c_uint64,
                           ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_int)]

    def call(roots, gmax, batched=False, max_root_chunk=0):
        c, g, n = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_int()
        lib.layout(roots, gmax, int(batched), max_root_chunk, ctypes.byref(c), ctypes.byref(g), ctypes.byref(n))
        return c.value, g.value, bool(n.value)
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
