"""The engine's normal sampler against the oracle's, on the host.

csrc/pc_rng.h is compiled for both the device and the host (IEEE add, multiply and divide
only, no contraction), so its host build evaluates exactly what the kernels do. Here it is
compiled with the engine's own ziggurat tables (pc::host_zig_tables, from libprocell.so)
and compared bit for bit with the oracle's independent restatement over two million draws:
the first attempt from the pair block (layer and wedge bits), the wedge test, the tail
beyond r (about 1 in 17,500 draws, so over a hundred here) and the restarts from the node's
private stream. A constant that differs between the two (a table size, r of the tail) shows
up here without a GPU.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "cuda-pro-cell_gb300", "csrc")


@pytest.fixture(scope="module")
def host_sampler(built, tmp_path_factory):
    from procell import _lib
    out = str(tmp_path_factory.mktemp("sampler") / "libhost_sampler.so")
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                    "-I" + CSRC, os.path.join(ROOT, "tests", "host_sampler.cpp"), "-o", out,
                    "-L" + libdir, "-lprocell", "-Wl,-rpath," + libdir], check=True)
    ctypes.CDLL(_lib.LIB_PATH, mode=ctypes.RTLD_GLOBAL)
    lib = ctypes.CDLL(out)
    lib.host_normals.restype = ctypes.c_int
    lib.host_normals.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64,
                                 ctypes.POINTER(ctypes.c_float)]
    return lib


@pytest.mark.parametrize("seed,root,first_parent", [(2024, 3, 0), (2 ** 63 + 11, 77, 10 ** 9)])
def test_device_sampler_on_host_equals_oracle(host_sampler, oracle_lib, seed, root, first_parent):
    n = 2_000_000
    z = np.zeros(n, np.float32)
    assert host_sampler.host_normals(seed, root, first_parent, n, z.ctypes.data_as(ctypes.POINTER(ctypes.c_float))) == 0
    o = oracle_lib.normals(seed=seed, root=root, first_parent=first_parent, count=n)
    bad = np.flatnonzero(z.view(np.uint32) != o.view(np.uint32))
    assert bad.size == 0, (bad[:5], z[bad[:5]], o[bad[:5]])
    # the tail beyond r was exercised
    assert np.sum(np.abs(z) > 4.0388498461095045227) > 20
