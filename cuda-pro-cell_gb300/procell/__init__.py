"""Python front end of the GB300 proliferation engine (libprocell.so).

    from procell import Engine
    eng = Engine()                       # a pc_context on cuda:0
    h = eng.simulate(bins, types, t_max=168, phi=None, seed=7)
    h.values, h.totals, h.per_type, h.stats

bins are (value, frequency) rows and types (ratio, mean, sd) rows, both in file order, as
in the reference's histogram and cell-type files.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import ProcellError

ZIG_LAYERS = 1024  # layers of the normal sampler's ziggurat (pc_rng.h kZigLayers)

__all__ = ["Engine", "Batch", "Result", "log_space", "rebin", "ProcellError", "format_histogram"]


@dataclass
class Result:
    values: np.ndarray      # float64 [V] ascending output value set
    totals: np.ndarray      # uint64 [V]
    per_type: np.ndarray    # uint64 [V, ntypes] (file order)
    stats: dict = field(default_factory=dict)


class Plan:
    """A prepared input resident in HBM (pc_plan). run() may be repeated."""

    def __init__(self, engine: "Engine", bins, types, t_max, phi=None, seed=0):
        self.engine = engine
        L = engine.L
        b, t = _lib.bins_numpy(bins), _lib.types_numpy(types)
        h = ctypes.c_void_p()
        rc = L.pc_plan_create(engine.ctx, b.ctypes.data_as(ctypes.POINTER(_lib.Bin)), len(b),
                              t.ctypes.data_as(ctypes.POINTER(_lib.CellType)), len(t),
                              float(t_max), 0.0 if phi is None else float(phi), int(seed),
                              ctypes.byref(h))
        engine._check(rc)
        self.handle = h

    def set_roots(self, begin, end):
        self.engine._check(self.engine.L.pc_plan_set_roots(self.engine.ctx, self.handle,
                                                           int(begin), int(end)))

    def run(self):
        self.engine._check(self.engine.L.pc_plan_run(self.engine.ctx, self.handle))

    def stats(self) -> dict:
        st = _lib.Stats()
        self.engine._check(self.engine.L.pc_plan_stats(self.engine.ctx, self.handle, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in _lib.Stats._fields_}

    def result(self) -> Result:
        h = _lib.Histogram()
        self.engine._check(self.engine.L.pc_plan_result(self.engine.ctx, self.handle, ctypes.byref(h)))
        try:
            return Result(*_lib.histogram_to_numpy(h))
        finally:
            self.engine.L.pc_histogram_free(ctypes.byref(h))

    def raw_counts(self) -> np.ndarray:
        L, n = self.engine.L, ctypes.c_uint64()
        dims = (ctypes.c_uint32 * 3)()
        self.engine._check(L.pc_plan_raw_counts(self.engine.ctx, self.handle, None, 0,
                                                ctypes.byref(n), dims))
        out = np.zeros(int(n.value), np.uint64)
        self.engine._check(L.pc_plan_raw_counts(
            self.engine.ctx, self.handle, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
            int(n.value), ctypes.byref(n), dims))
        return out.reshape(dims[0], dims[1], dims[2])

    def close(self):
        if getattr(self, "handle", None):
            self.engine.L.pc_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def instance_array(instances):
    """A pc_instance array of (bins, types, t_max, phi, seed) tuples or dicts, and the numpy
    arrays it points into (keep them alive while the array is used)."""
    keep = []
    arr = (_lib.Instance * max(1, len(instances)))()
    for i, inst in enumerate(instances):
        if isinstance(inst, dict):
            bins, types, t_max = inst["bins"], inst["types"], inst["t_max"]
            phi, seed = inst.get("phi"), inst.get("seed", 0)
        else:
            bins, types, t_max, phi, seed = inst
        b, t = _lib.bins_numpy(bins), _lib.types_numpy(types)
        keep += [b, t]
        arr[i].bins = b.ctypes.data_as(ctypes.POINTER(_lib.Bin))
        arr[i].n_bins = len(b)
        arr[i].types = t.ctypes.data_as(ctypes.POINTER(_lib.CellType))
        arr[i].n_types = len(t)
        arr[i].reserved = 0
        arr[i].t_max = float(t_max)
        arr[i].phi = 0.0 if phi is None else float(phi)
        arr[i].seed = int(seed)
    return arr, keep


class Batch:
    """Many independent instances in one run (pc_batch). Each instance is a dict or tuple
    (bins, types, t_max, phi, seed); bins may be (values, frequencies) numpy arrays."""

    def __init__(self, engine: "Engine", instances):
        self.engine = engine
        arr, self._keep = instance_array(instances)
        h = ctypes.c_void_p()
        engine._check(engine.L.pc_batch_create(engine.ctx, arr, len(instances), ctypes.byref(h)))
        self.handle = h
        self._keep = []  # the library copied the inputs
        self.size = len(instances)

    def run(self):
        self.engine._check(self.engine.L.pc_batch_run(self.engine.ctx, self.handle))

    def stats(self) -> dict:
        st = _lib.Stats()
        self.engine._check(self.engine.L.pc_batch_stats(self.engine.ctx, self.handle, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in _lib.Stats._fields_}

    def result(self, i: int) -> Result:
        h = _lib.Histogram()
        self.engine._check(self.engine.L.pc_batch_result(self.engine.ctx, self.handle, int(i), ctypes.byref(h)))
        try:
            return Result(*_lib.histogram_to_numpy(h))
        finally:
            self.engine.L.pc_histogram_free(ctypes.byref(h))

    def set_types(self, types):
        """New cell types for every instance: a TYPE_DTYPE array (or rows of (ratio, mean,
        sd)) concatenated in instance order, each instance with its original type count."""
        t = np.ascontiguousarray(types if isinstance(types, np.ndarray) and types.dtype == _lib.TYPE_DTYPE
                                 else _lib.types_numpy(types))
        self.engine._check(self.engine.L.pc_batch_set_types(self.engine.ctx, self.handle,
                                                            t.ctypes.data_as(ctypes.POINTER(_lib.CellType))))

    def totals(self):
        """(offsets [n + 1], totals): instance i's merged counts are totals[offsets[i]:offsets[i + 1]]."""
        L = self.engine.L
        off = np.zeros(self.size + 1, np.uint64)
        U = ctypes.POINTER(ctypes.c_uint64)
        self.engine._check(L.pc_batch_totals(self.engine.ctx, self.handle, None, 0, off.ctypes.data_as(U)))
        out = np.zeros(int(off[-1]), np.uint64)
        self.engine._check(L.pc_batch_totals(self.engine.ctx, self.handle, out.ctypes.data_as(U), len(out), None))
        return off, out

    def raw_counts(self, i: int) -> np.ndarray:
        L, n = self.engine.L, ctypes.c_uint64()
        dims = (ctypes.c_uint32 * 3)()
        self.engine._check(L.pc_batch_raw_counts(self.engine.ctx, self.handle, int(i), None, 0,
                                                 ctypes.byref(n), dims))
        out = np.zeros(int(n.value), np.uint64)
        self.engine._check(L.pc_batch_raw_counts(
            self.engine.ctx, self.handle, int(i), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
            int(n.value), ctypes.byref(n), dims))
        return out.reshape(dims[0], dims[1], dims[2])

    def close(self):
        if getattr(self, "handle", None):
            self.engine.L.pc_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Engine:
    def __init__(self, device: int = 0):
        self.L = _lib.load()
        ctx = ctypes.c_void_p()
        rc = self.L.pc_create(ctypes.byref(ctx), int(device))
        if rc != 0:
            raise ProcellError(rc, self.L.pc_last_error(None).decode())
        self.ctx = ctx

    def _check(self, rc):
        if rc != 0:
            raise ProcellError(rc, self.L.pc_last_error(self.ctx).decode())

    def set_stream(self, stream_handle: int):
        """Run on an existing cudaStream_t (e.g. torch.cuda.current_stream().cuda_stream).
        Handle 0, torch's default stream, is the legacy default stream (cudaStreamLegacy)."""
        h = int(stream_handle) or 1
        self._check(self.L.pc_set_stream(self.ctx, ctypes.c_void_p(h)))

    def set_option(self, name: str, value: float):
        self._check(self.L.pc_set_option(self.ctx, name.encode(), float(value)))

    def plan(self, bins, types, t_max, phi=None, seed=0) -> Plan:
        return Plan(self, bins, types, t_max, phi, seed)

    def autotune(self, target, repeats: int = 2) -> dict:
        """Time every sweep configuration and driver on a Plan or Batch; the context keeps
        the fastest (results are identical under all of them)."""
        t = _lib.Tuning()
        fn = self.L.pc_batch_autotune if isinstance(target, Batch) else self.L.pc_autotune
        self._check(fn(self.ctx, target.handle, int(repeats), ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in _lib.Tuning._fields_}

    def batch(self, instances) -> Batch:
        return Batch(self, instances)

    def simulate_batch(self, instances) -> list:
        """pc_simulate_batch: every instance's merged histogram (host inputs in, host results
        out), as a list of Result."""
        arr, keep = instance_array(instances)
        n = len(instances)
        hs = (_lib.Histogram * max(1, n))()
        self._check(self.L.pc_simulate_batch(self.ctx, arr, n, hs))
        out = []
        try:
            for i in range(n):
                out.append(Result(*_lib.histogram_to_numpy(hs[i])))
        finally:
            for i in range(n):
                self.L.pc_histogram_free(ctypes.byref(hs[i]))
        del keep
        return out

    def simulate(self, bins, types, t_max, phi=None, seed=0, root_begin=None, root_end=None) -> Result:
        """pc_simulate (pc_simulate_shard for a range of initial cells): one input's merged
        histogram, host arrays in and out, in one library call."""
        b, t = _lib.bins_numpy(bins), _lib.types_numpy(types)
        h = _lib.Histogram()
        args = (self.ctx, b.ctypes.data_as(ctypes.POINTER(_lib.Bin)), len(b),
                t.ctypes.data_as(ctypes.POINTER(_lib.CellType)), len(t), float(t_max),
                0.0 if phi is None else float(phi), int(seed))
        if root_begin is not None or root_end is not None:
            total = int(b["frequency"].sum())
            rc = self.L.pc_simulate_shard(*args, int(root_begin or 0), total if root_end is None else int(root_end),
                                          ctypes.byref(h))
        else:
            rc = self.L.pc_simulate(*args, ctypes.byref(h))
        try:
            self._check(rc)
            return Result(*_lib.histogram_to_numpy(h))
        finally:
            self.L.pc_histogram_free(ctypes.byref(h))

    def get_option(self, name: str) -> float:
        v = ctypes.c_double()
        self._check(self.L.pc_get_option(self.ctx, name.encode(), ctypes.byref(v)))
        return v.value

    def peak(self, kind: str) -> float:
        """Measured lane-operations/s of one pipe: "fp64" / "fp32" FMA, "int32" multiply-add."""
        v = ctypes.c_double()
        self._check(self.L.pc_debug_peak(self.ctx, {"fp64": 0, "fp32": 1, "int32": 2}[kind], ctypes.byref(v)))
        return v.value

    def philox(self, ctrs: np.ndarray, key) -> np.ndarray:
        c = np.ascontiguousarray(ctrs, dtype=np.uint32).reshape(-1, 4)
        out = np.zeros_like(c)
        k = (ctypes.c_uint32 * 2)(*key)
        self._check(self.L.pc_debug_philox(self.ctx, c.ctypes.data_as(_lib.U32P), c.shape[0], k,
                                           out.ctypes.data_as(_lib.U32P)))
        return out

    def normals(self, seed, root, first_parent, count) -> np.ndarray:
        z = np.zeros(int(count), np.float32)
        self._check(self.L.pc_debug_normals(self.ctx, int(seed), int(root), int(first_parent),
                                            int(count), z.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return z

    def tables(self):
        k = np.zeros(ZIG_LAYERS, np.uint32)
        w = np.zeros(ZIG_LAYERS, np.uint32)
        f = np.zeros(ZIG_LAYERS + 1, np.uint32)
        self._check(self.L.pc_debug_tables(self.ctx, k.ctypes.data_as(_lib.U32P),
                                           w.ctypes.data_as(_lib.U32P), f.ctypes.data_as(_lib.U32P)))
        return k, w.view(np.float32), f.view(np.float32)

    def close(self):
        if getattr(self, "ctx", None):
            self.L.pc_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def log_space(start: float, end: float, n: int, base: float = 10.0) -> np.ndarray:
    """pc_log_space: the reference's logarithmic bin edges."""
    L = _lib.load()
    e = np.zeros(int(n), np.float64)
    rc = L.pc_log_space(float(start), float(end), int(n), float(base), e.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    if rc != 0:
        raise ProcellError(rc, "invalid log_space arguments")
    return e


def rebin(values, counts, lower: float, upper: float, n_bins: int):
    """pc_rebin: an ascending histogram summed into log_space(lower, upper, n_bins, 10)."""
    L = _lib.load()
    v = np.ascontiguousarray(values, np.float64)
    c = np.ascontiguousarray(counts, np.uint64)
    e = np.zeros(int(n_bins), np.float64)
    out = np.zeros(int(n_bins), np.uint64)
    rc = L.pc_rebin(v.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), c.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                    len(v), float(lower), float(upper), int(n_bins), e.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                    out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
    if rc != 0:
        raise ProcellError(rc, "rebin: values out of order or above the last edge, or invalid edges")
    return e, out


def format_histogram(values, totals, per_type, track_ratio: bool) -> str:
    """The output text of the reference's io::save_fluorescences (src/io/parser.cu:187-217)."""
    out = []
    for i, v in enumerate(values):
        if int(totals[i]) == 0:
            continue
        row = "%.10g\t%d" % (v, int(totals[i]))
        if track_ratio:
            row += "".join("\t%d" % int(c) for c in per_type[i])
        out.append(row + "\n")
    return "".join(out)
