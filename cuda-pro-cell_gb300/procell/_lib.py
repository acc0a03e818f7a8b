"""ctypes binding of libprocell.so (include/procell.h).

The library must have been built (cuda-pro-cell_gb300/build.py); loading fails loudly
otherwise. There is no CPU fallback: every simulation runs on the GPU.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# PROCELL_LIB selects another build of the library (e.g. a tuning variant).
LIB_PATH = os.environ.get("PROCELL_LIB") or os.path.join(PKG, "build", "libprocell.so")
CLI_PATH = os.path.join(PKG, "build", "procell")

PC_OK = 0
ERRORS = {1: "PC_ERR_INVALID", 2: "PC_ERR_CUDA", 3: "PC_ERR_NOMEM", 4: "PC_ERR_DEPTH",
          5: "PC_ERR_UNSUPPORTED", 6: "PC_ERR_IO", 7: "PC_ERR_INTERNAL"}


class Bin(ctypes.Structure):
    _fields_ = [("value", ctypes.c_double), ("frequency", ctypes.c_uint64)]


class CellType(ctypes.Structure):
    _fields_ = [("ratio", ctypes.c_double), ("mean", ctypes.c_double), ("sd", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [("roots", ctypes.c_uint64), ("divisions", ctypes.c_uint64),
                ("leaves", ctypes.c_uint64), ("uncounted", ctypes.c_uint64),
                ("vanished", ctypes.c_uint64), ("max_generation", ctypes.c_uint32),
                ("sweeps", ctypes.c_uint32), ("root_sweeps", ctypes.c_uint32),
                ("kernel_launches", ctypes.c_uint32), ("device_ms", ctypes.c_double),
                ("divide_ms", ctypes.c_double), ("h2d_bytes", ctypes.c_uint64),
                ("d2h_bytes", ctypes.c_uint64)]


class Histogram(ctypes.Structure):
    _fields_ = [("n_values", ctypes.c_uint64), ("n_types", ctypes.c_uint32),
                ("values", ctypes.POINTER(ctypes.c_double)),
                ("totals", ctypes.POINTER(ctypes.c_uint64)),
                ("per_type", ctypes.POINTER(ctypes.c_uint64)), ("stats", Stats)]


class Instance(ctypes.Structure):
    _fields_ = [("bins", ctypes.POINTER(Bin)), ("n_bins", ctypes.c_uint64),
                ("types", ctypes.POINTER(CellType)), ("n_types", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32), ("t_max", ctypes.c_double), ("phi", ctypes.c_double),
                ("seed", ctypes.c_uint64)]


class Tuning(ctypes.Structure):
    _fields_ = [("config", ctypes.c_int32), ("driver", ctypes.c_int32), ("threads", ctypes.c_int32),
                ("cells_per_lane", ctypes.c_int32), ("global_hist", ctypes.c_int32),
                ("candidates", ctypes.c_int32), ("ms", ctypes.c_double), ("ms_default", ctypes.c_double)]


# (name, restype, argtypes) of every exported symbol of include/procell.h
VP, U32P, U64P = ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint64)
SIGNATURES = [
    ("pc_create", ctypes.c_int, [ctypes.POINTER(VP), ctypes.c_int]),
    ("pc_destroy", None, [VP]),
    ("pc_last_error", ctypes.c_char_p, [VP]),
    ("pc_version", ctypes.c_char_p, []),
    ("pc_set_stream", ctypes.c_int, [VP, VP]),
    ("pc_set_option", ctypes.c_int, [VP, ctypes.c_char_p, ctypes.c_double]),
    ("pc_plan_create", ctypes.c_int, [VP, ctypes.POINTER(Bin), ctypes.c_uint64,
                                      ctypes.POINTER(CellType), ctypes.c_uint32, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_uint64, ctypes.POINTER(VP)]),
    ("pc_plan_set_roots", ctypes.c_int, [VP, VP, ctypes.c_uint64, ctypes.c_uint64]),
    ("pc_plan_run", ctypes.c_int, [VP, VP]),
    ("pc_plan_stats", ctypes.c_int, [VP, VP, ctypes.POINTER(Stats)]),
    ("pc_plan_result", ctypes.c_int, [VP, VP, ctypes.POINTER(Histogram)]),
    ("pc_plan_raw_counts", ctypes.c_int, [VP, VP, U64P, ctypes.c_uint64, U64P, U32P]),
    ("pc_plan_destroy", None, [VP]),
    ("pc_simulate", ctypes.c_int, [VP, ctypes.POINTER(Bin), ctypes.c_uint64,
                                   ctypes.POINTER(CellType), ctypes.c_uint32, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_uint64, ctypes.POINTER(Histogram)]),
    ("pc_histogram_free", None, [ctypes.POINTER(Histogram)]),
    ("pc_simulate_shard", ctypes.c_int, [VP, ctypes.POINTER(Bin), ctypes.c_uint64, ctypes.POINTER(CellType),
                                         ctypes.c_uint32, ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                         ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(Histogram)]),
    ("pc_histogram_accumulate", ctypes.c_int, [ctypes.POINTER(Histogram), ctypes.POINTER(Histogram)]),
    ("pc_batch_create", ctypes.c_int, [VP, ctypes.POINTER(Instance), ctypes.c_uint32, ctypes.POINTER(VP)]),
    ("pc_batch_run", ctypes.c_int, [VP, VP]),
    ("pc_batch_stats", ctypes.c_int, [VP, VP, ctypes.POINTER(Stats)]),
    ("pc_batch_size", ctypes.c_uint32, [VP]),
    ("pc_batch_result", ctypes.c_int, [VP, VP, ctypes.c_uint32, ctypes.POINTER(Histogram)]),
    ("pc_batch_raw_counts", ctypes.c_int, [VP, VP, ctypes.c_uint32, U64P, ctypes.c_uint64, U64P, U32P]),
    ("pc_batch_set_types", ctypes.c_int, [VP, VP, ctypes.POINTER(CellType)]),
    ("pc_batch_totals", ctypes.c_int, [VP, VP, U64P, ctypes.c_uint64, U64P]),
    ("pc_batch_destroy", None, [VP]),
    ("pc_simulate_batch", ctypes.c_int, [VP, ctypes.POINTER(Instance), ctypes.c_uint32,
                                         ctypes.POINTER(Histogram)]),
    ("pc_autotune", ctypes.c_int, [VP, VP, ctypes.c_uint32, ctypes.POINTER(Tuning)]),
    ("pc_batch_autotune", ctypes.c_int, [VP, VP, ctypes.c_uint32, ctypes.POINTER(Tuning)]),
    ("pc_smooth_create", ctypes.c_int, [VP, ctypes.POINTER(Bin), ctypes.c_uint64, ctypes.c_uint32,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_uint32,
                                        ctypes.c_uint64, ctypes.POINTER(VP)]),
    ("pc_smooth_info", ctypes.c_int, [VP, U64P, U32P, U64P]),
    ("pc_smooth_values", ctypes.c_int, [VP, ctypes.POINTER(ctypes.c_double)]),
    ("pc_smooth_forward", ctypes.c_int, [VP, VP, VP, ctypes.c_uint32, VP]),
    ("pc_smooth_backward", ctypes.c_int, [VP, VP, VP, ctypes.c_uint32, VP, VP]),
    ("pc_smooth_jacobian", ctypes.c_int, [VP, VP, VP, ctypes.c_uint32, VP, VP]),
    ("pc_smooth_gauss_newton", ctypes.c_int, [VP, VP, VP, ctypes.c_uint32, VP, VP, VP, VP]),
    ("pc_smooth_sync", ctypes.c_int, [VP]),
    ("pc_smooth_destroy", None, [VP]),
    ("pc_log_space", ctypes.c_int, [ctypes.c_double, ctypes.c_double, ctypes.c_uint64, ctypes.c_double,
                                    ctypes.POINTER(ctypes.c_double)]),
    ("pc_rebin", ctypes.c_int, [ctypes.POINTER(ctypes.c_double), U64P, ctypes.c_uint64, ctypes.c_double,
                                ctypes.c_double, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double), U64P]),
    ("pc_load_histogram", ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.POINTER(Bin)), U64P]),
    ("pc_load_cell_types", ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.POINTER(CellType)), U32P]),
    ("pc_write_histogram", ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(Histogram), ctypes.c_int]),
    ("pc_free", None, [VP]),
    ("pc_simulate_noalloc", ctypes.c_int, [ctypes.POINTER(Bin), ctypes.c_uint64, ctypes.POINTER(CellType),
                                           ctypes.c_uint32, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_uint64, VP, U64P, ctypes.c_uint64, U32P,
                                           ctypes.POINTER(Stats), ctypes.c_char_p, ctypes.c_size_t]),
    ("pc_debug_barrier", ctypes.c_int, [VP, ctypes.c_int, ctypes.c_double, U32P, U32P]),
    ("pc_debug_philox", ctypes.c_int, [VP, U32P, ctypes.c_uint64, U32P, U32P]),
    ("pc_debug_peak", ctypes.c_int, [VP, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    ("pc_get_option", ctypes.c_int, [VP, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double)]),
    ("pc_debug_normals", ctypes.c_int, [VP, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64,
                                        ctypes.c_uint64, ctypes.POINTER(ctypes.c_float)]),
    ("pc_debug_tables", ctypes.c_int, [VP, U32P, U32P, U32P]),
]

_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libprocell.so is not built ({LIB_PATH}); run "
                               "`python cuda-pro-cell_gb300/build.py` first")
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class ProcellError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def bins_array(bins):
    arr = (Bin * max(1, len(bins)))()
    for i, (v, f) in enumerate(bins):
        arr[i].value = float(v)
        arr[i].frequency = int(f)
    return arr


def types_array(types):
    arr = (CellType * max(1, len(types)))()
    for i, (r, m, s) in enumerate(types):
        arr[i].ratio, arr[i].mean, arr[i].sd = float(r), float(m), float(s)
    return arr


def histogram_to_numpy(h: Histogram):
    nv, nt = int(h.n_values), int(h.n_types)
    values = np.ctypeslib.as_array(h.values, shape=(max(1, nv),))[:nv].copy()
    totals = np.ctypeslib.as_array(h.totals, shape=(max(1, nv),))[:nv].copy()
    per = np.ctypeslib.as_array(h.per_type, shape=(max(1, nv * nt),))[:nv * nt].copy().reshape(nv, nt)
    st = h.stats
    stats = {k: getattr(st, k) for k, _ in Stats._fields_}
    return values, totals.astype(np.uint64, copy=False), per.astype(np.uint64, copy=False), stats


BIN_DTYPE = np.dtype([("value", "<f8"), ("frequency", "<u8")])
TYPE_DTYPE = np.dtype([("ratio", "<f8"), ("mean", "<f8"), ("sd", "<f8")])


def bins_numpy(bins) -> np.ndarray:
    """(value, frequency) rows as a pc_bin array; accepts a list of pairs or a (values,
    frequencies) pair of numpy arrays, or a pc_bin array itself."""
    if isinstance(bins, np.ndarray) and bins.dtype == BIN_DTYPE:
        return np.ascontiguousarray(bins)
    if isinstance(bins, tuple) and len(bins) == 2 and isinstance(bins[0], np.ndarray):
        out = np.empty(len(bins[0]), BIN_DTYPE)
        out["value"], out["frequency"] = bins[0], bins[1]
        return out
    out = np.empty(len(bins), BIN_DTYPE)
    for i, (v, f) in enumerate(bins):
        out[i] = (float(v), int(f))
    return out


def types_numpy(types) -> np.ndarray:
    out = np.empty(len(types), TYPE_DTYPE)
    for i, (r, m, sd) in enumerate(types):
        out[i] = (float(r), float(m), float(sd))
    return out

