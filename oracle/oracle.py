"""Test infrastructure only: ctypes wrapper of the CPU oracle (oracle/liboracle.so).

Imported by the test suite, the smoke check and the benchmark's CPU-baseline leg, as the
CPU restatement the GPU engine is compared against; the engine itself never loads this
library.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "liboracle.so")
ZIG_LAYERS = 1024  # layers of the ziggurat (oracle.cpp kLayers)

_lib = None


def build() -> str:
    """Compile the oracle with its Makefile (a few seconds)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        c_dp, c_u64p = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint64)
        L.oracle_simulate.restype = ctypes.c_void_p
        L.oracle_simulate.argtypes = [c_dp, c_u64p, ctypes.c_uint64, c_dp, c_dp, c_dp,
                                      ctypes.c_uint32, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64,
                                      ctypes.c_uint64, ctypes.c_int]
        L.oracle_last_error.restype = ctypes.c_char_p
        L.oracle_result_nvalues.restype = ctypes.c_uint64
        L.oracle_result_nvalues.argtypes = [ctypes.c_void_p]
        L.oracle_result_ntypes.restype = ctypes.c_uint32
        L.oracle_result_ntypes.argtypes = [ctypes.c_void_p]
        L.oracle_result_copy.argtypes = [ctypes.c_void_p, c_dp, c_u64p, c_u64p, c_u64p]
        L.oracle_result_free.argtypes = [ctypes.c_void_p]
        u32p = ctypes.POINTER(ctypes.c_uint32)
        L.oracle_philox.argtypes = [u32p, u32p, u32p]
        L.oracle_tables.argtypes = [u32p, u32p, u32p]
        L.oracle_normals.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64,
                                     ctypes.c_uint64, ctypes.POINTER(ctypes.c_float)]
        L.oracle_tau.restype = ctypes.c_double
        L.oracle_tau.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64,
                                 ctypes.c_uint32, ctypes.c_double, ctypes.c_double]
        L.oracle_smooth.restype = ctypes.c_int
        L.oracle_smooth.argtypes = [c_dp, c_u64p, ctypes.c_uint64, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_int, ctypes.c_double, ctypes.c_uint32, ctypes.c_uint64, c_dp,
                                    ctypes.c_uint32, ctypes.c_uint32, c_dp, c_dp, c_dp, ctypes.c_uint64,
                                    c_u64p, ctypes.c_int]
        L.oracle_expf.restype = ctypes.c_float
        L.oracle_expf.argtypes = [ctypes.c_float]
        L.oracle_logf.restype = ctypes.c_float
        L.oracle_logf.argtypes = [ctypes.c_float]
        _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


@dataclass
class OracleResult:
    values: np.ndarray     # float64 [V], ascending: the output value set
    totals: np.ndarray     # uint64 [V]
    per_type: np.ndarray   # uint64 [V, ntypes], file order
    stats: dict = field(default_factory=dict)


def _ptr(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def simulate(bins, types, t_max, phi=None, seed=0, root_begin=0, root_end=None,
             nthreads=0) -> OracleResult:
    """Run the oracle on histogram rows `bins` [(value, freq), ...] and `types`
    [(ratio, mean, sd), ...], both in file order. phi=None selects the automatic
    threshold (minimum value with a nonzero frequency)."""
    L = lib()
    b = np.asarray(bins, dtype=np.float64).reshape(-1, 2) if len(bins) else np.zeros((0, 2))
    values = np.ascontiguousarray(b[:, 0], dtype=np.float64)
    freqs = np.ascontiguousarray([int(f) for _, f in bins] if len(bins) else [], dtype=np.uint64)
    t = np.asarray(types, dtype=np.float64).reshape(-1, 3)
    ratio, mean, sd = (np.ascontiguousarray(t[:, i]) for i in range(3))
    end = (1 << 64) - 1 if root_end is None else int(root_end)
    h = L.oracle_simulate(_ptr(values, ctypes.c_double), _ptr(freqs, ctypes.c_uint64),
                          len(values), _ptr(ratio, ctypes.c_double), _ptr(mean, ctypes.c_double),
                          _ptr(sd, ctypes.c_double), len(ratio), float(t_max),
                          float(phi) if phi is not None else 0.0, 0 if phi is None else 1,
                          int(seed), int(root_begin), end, int(nthreads))
    if not h:
        raise OracleError(L.oracle_last_error().decode())
    try:
        nv, nt = L.oracle_result_nvalues(h), L.oracle_result_ntypes(h)
        vals = np.zeros(nv, np.float64)
        tot = np.zeros(nv, np.uint64)
        per = np.zeros((nv, nt), np.uint64)
        st = np.zeros(6, np.uint64)
        L.oracle_result_copy(h, _ptr(vals, ctypes.c_double), _ptr(tot, ctypes.c_uint64),
                             _ptr(per, ctypes.c_uint64), _ptr(st, ctypes.c_uint64))
    finally:
        L.oracle_result_free(h)
    keys = ["roots", "divisions", "leaves", "uncounted", "vanished", "max_gen"]
    return OracleResult(vals, tot, per, {k: int(v) for k, v in zip(keys, st)})


def smooth(bins, t_max, phi, h, paths, seed, params, grad_expected=None, nthreads=0):
    """The smoothed form in C++ (the restatement of smooth_ref.forward_backward, FP64,
    multi-threaded): (expected [C][V], gradient [C][K][3] or None, values [V])."""
    L = lib()
    b = np.asarray(bins, dtype=np.float64).reshape(-1, 2) if len(bins) else np.zeros((0, 2))
    values = np.ascontiguousarray(b[:, 0], dtype=np.float64)
    freqs = np.ascontiguousarray([int(f) for _, f in bins] if len(bins) else [], dtype=np.uint64)
    P = np.ascontiguousarray(params, dtype=np.float64)
    C, K = P.shape[0], P.shape[1]
    nv = ctypes.c_uint64()
    args = (_ptr(values, ctypes.c_double), _ptr(freqs, ctypes.c_uint64), len(values), float(t_max),
            float(phi) if phi else 0.0, 1 if phi else 0, float(h), int(paths), int(seed),
            _ptr(P, ctypes.c_double), C, K)
    dummy = np.zeros(1)
    L.oracle_smooth(*args, None, _ptr(dummy, ctypes.c_double), None, 0, ctypes.byref(nv), 1)
    V = int(nv.value)
    E = np.zeros((C, V))
    G = np.zeros((C, K, 3)) if grad_expected is not None else None
    gE = None if grad_expected is None else np.ascontiguousarray(grad_expected, dtype=np.float64)
    rc = L.oracle_smooth(*args, None if gE is None else _ptr(gE, ctypes.c_double), _ptr(E, ctypes.c_double),
                         None if G is None else _ptr(G, ctypes.c_double), V, ctypes.byref(nv), int(nthreads))
    if rc != 0:
        raise OracleError("oracle_smooth: value set larger than expected or too many lineages")
    return E, G


def philox(ctr, key):
    L = lib()
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    L.oracle_philox(c, k, o)
    return list(o)


def tables():
    L = lib()
    k = np.zeros(ZIG_LAYERS, np.uint32)
    w = np.zeros(ZIG_LAYERS, np.uint32)
    f = np.zeros(ZIG_LAYERS + 1, np.uint32)
    L.oracle_tables(_ptr(k, ctypes.c_uint32), _ptr(w, ctypes.c_uint32), _ptr(f, ctypes.c_uint32))
    return k, w.view(np.float32), f.view(np.float32)


def normals(seed, root, first_parent, count):
    z = np.zeros(int(count), np.float32)
    lib().oracle_normals(int(seed), int(root), int(first_parent), int(count),
                         _ptr(z, ctypes.c_float))
    return z


def tau(seed, root, parent, child, mean, sd):
    return lib().oracle_tau(int(seed), int(root), int(parent), int(child), float(mean), float(sd))


def expf(x):
    return lib().oracle_expf(float(x))


def logf(u):
    return lib().oracle_logf(float(u))


def format_histogram(res: OracleResult, track_ratio: bool) -> str:
    """The reference's output text (io::save_fluorescences, src/io/parser.cu:187-217):
    rows with a nonzero count, ascending value, `%.10g`, tab separated."""
    out = []
    for i, v in enumerate(res.values):
        if int(res.totals[i]) == 0:
            continue
        row = "%.10g\t%d" % (v, int(res.totals[i]))
        if track_ratio:
            row += "".join("\t%d" % int(c) for c in res.per_type[i])
        out.append(row + "\n")
    return "".join(out)
