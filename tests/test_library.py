"""CPU checks of the drop-in boundary: libprocell.so builds for sm_103a, loads, exports
every symbol include/procell.h declares, and the CLI honours the reference's flag
contract (src/io/cmdargs.cpp:11-375) before any GPU work starts."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "procell.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(pc_\w+)\s*\(", text, re.M)))


def test_header_symbols_exported(built):
    from procell import _lib
    lib = ctypes.CDLL(_lib.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert set(syms) == bound, set(syms) ^ bound


def test_create_without_gpu_fails_cleanly(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from procell import Engine, ProcellError
    with pytest.raises(ProcellError, match="PC_ERR_CUDA"):
        Engine(0)


def test_version_string(built):
    from procell import _lib
    assert b"sm_103a" in _lib.load().pc_version()


def run_cli(args, cwd=None):
    from procell import _lib
    return subprocess.run([_lib.CLI_PATH, *args], capture_output=True, text=True, cwd=cwd)


@pytest.mark.parametrize("args,code,msg", [
    (["-x"], 1, "Invalid option -x\n"),
    (["-h"], 1, "Option --histogram (-h) requires a filename\n"),
    (["-h", "a", "-h", "b"], 1, "Option --histogram (-h) already given\n"),
    (["-c", "a", "--cell-types", "b"], 1, "Option --cell-types (-c) already given\n"),
    (["-o"], 1, "Option --output-histogram (-o) requires a filename\n"),
    (["-t", "-3"], 1, "Option --time-max (-t) requires an integer value >= 0\n"),
    (["-t"], 1, "Option --time-max (-t) requires an integer value >= 0\n"),
    (["-t", "1", "-t", "2"], 1, "Option --time-max (-t) already given\n"),
    (["-p", "0"], 1, "Option --phi-min (-p) requires a double value > 0\n"),
    (["-p", "abc"], 1, "Option --phi-min (-p) requires a double value > 0\n"),
    (["-d", "0"], 1, "Option --tree-depth (-d) requires an integer value >= 1 && <= 23\n"),
    (["-d", "24"], 1, "Option --tree-depth (-d) requires an integer value >= 1 && <= 23\n"),
    (["-d"], 1, "Option --tree-depth (-d) requires an integer value >= 1\n"),
    (["-r", "-r"], 1, "Option --track-ratio (-r) already given\n"),
    ([], 1, "The following missing arguments are required:\n--histogram (-h)\n"
            "--cell-types (-c)\n--t-max (-t)\n"),
    (["-h", "x", "-t", "1"], 1, "The following missing arguments are required:\n--cell-types (-c)\n"),
])
def test_cli_flag_errors(built, args, code, msg):
    r = run_cli(args)
    assert r.returncode == code
    assert r.stdout == msg


def test_cli_help(built):
    r = run_cli(["--help"])
    assert r.returncode == 0 and "usage: procell" in r.stdout


def test_cli_missing_file(built, tmp_path):
    r = run_cli(["-h", str(tmp_path / "nope"), "-c", "x", "-t", "1"])
    assert r.returncode == 1 and "cannot open histogram file" in r.stdout


def test_cli_bad_ratio_sum(built, tmp_path):
    h = tmp_path / "h.txt"
    c = tmp_path / "c.txt"
    h.write_text("4 10\n")
    c.write_text("0.5 10 1\n0.4 20 1\n")
    r = run_cli(["-h", str(h), "-c", str(c), "-t", "1"])
    assert r.returncode == 1
    assert r.stdout == "ERROR: proportion distribution of cell types does not sum to 1, aborting.\n"


def test_loaders_follow_stream_semantics(built, tmp_path):
    from procell import _lib
    L = _lib.load()
    p = tmp_path / "h.txt"
    # `in >> double >> uint64` stops at the first token that does not parse
    p.write_text("1.5 3\n  2e3\t0\n7 4 x 9 9\n")
    out = ctypes.POINTER(_lib.Bin)()
    n = ctypes.c_uint64()
    assert L.pc_load_histogram(str(p).encode(), ctypes.byref(out), ctypes.byref(n)) == 0
    rows = [(out[i].value, out[i].frequency) for i in range(n.value)]
    L.pc_free(out)
    assert rows == [(1.5, 3), (2000.0, 0), (7.0, 4)]
    t = tmp_path / "t.txt"
    t.write_text("0.53 48.33 21.6\n0.47 -1 -1\n")
    tout = ctypes.POINTER(_lib.CellType)()
    nt = ctypes.c_uint32()
    assert L.pc_load_cell_types(str(t).encode(), ctypes.byref(tout), ctypes.byref(nt)) == 0
    got = [(tout[i].ratio, tout[i].mean, tout[i].sd) for i in range(nt.value)]
    L.pc_free(tout)
    assert got == [(0.53, 48.33, 21.6), (0.47, -1.0, -1.0)]


def test_writer_matches_reference_format(built, tmp_path):
    from procell import _lib, format_histogram
    L = _lib.load()
    vals = np.array([1e-05, 0.5, 3.0, 123456789012.5, 7.25], np.float64)
    tot = np.array([2, 0, 5, 1, 9], np.uint64)
    per = np.array([[1, 1], [0, 0], [5, 0], [0, 1], [4, 5]], np.uint64)
    h = _lib.Histogram()
    h.n_values, h.n_types = len(vals), 2
    h.values = vals.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    h.totals = tot.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
    h.per_type = per.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
    for track in (0, 1):
        path = tmp_path / f"o{track}.txt"
        assert L.pc_write_histogram(str(path).encode(), ctypes.byref(h), track) == 0
        assert path.read_text() == format_histogram(vals, tot, per, bool(track))
    assert (tmp_path / "o0.txt").read_text() == "1e-05\t2\n3\t5\n1.23456789e+11\t1\n7.25\t9\n"


def test_log_space_and_rebin_follow_the_reference(built):
    """pc_log_space / pc_rebin against a restatement of the reference's helpers
    (src/utils/util.cu:76-138): exponents ceil(log10(lower))..ceil(log10(upper)) in equal steps,
    each value into the first bin whose edge is >= it."""
    import math
    from procell import ProcellError, log_space, rebin
    e = log_space(3.0, 2e4, 6, 10.0)
    lo, hi = math.ceil(math.log10(3.0)), math.ceil(math.log10(2e4))
    want = [10.0 ** (lo + (hi - lo) / 5 * i) for i in range(5)] + [10.0 ** hi]
    assert np.allclose(e, want, rtol=1e-15)
    vals = np.array([0.5, 1.0, 9.9, 10.0, 10.5, 99.0, 1000.0])
    cnts = np.array([1, 2, 3, 4, 5, 6, 7], np.uint64)
    edges, out = rebin(vals, cnts, 1.0, 1000.0, 4)
    assert np.allclose(edges, [1.0, 10.0, 100.0, 1000.0])
    assert out.tolist() == [3, 7, 11, 7]  # 0.5,1 | 9.9,10 | 10.5,99 | 1000
    with pytest.raises(ProcellError):
        rebin(np.array([5000.0]), np.array([1], np.uint64), 1.0, 1000.0, 4)
    with pytest.raises(ProcellError):
        rebin(np.array([5.0, 2.0]), np.array([1, 1], np.uint64), 1.0, 1000.0, 4)


def _histogram(values, totals, per_type, **stats):
    from procell import _lib
    v = np.ascontiguousarray(values, dtype=np.float64)
    t = np.ascontiguousarray(totals, dtype=np.uint64)
    p = np.ascontiguousarray(per_type, dtype=np.uint64)
    h = _lib.Histogram()
    h.n_values, h.n_types = len(v), p.shape[1]
    h.values = v.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    h.totals = t.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
    h.per_type = p.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
    for k, x in stats.items():
        setattr(h.stats, k, x)
    return h, (v, t, p)


def test_histogram_accumulate(built):
    """pc_histogram_accumulate (host only): shard histograms add element-wise; statistics
    add (max_generation: the larger); a different value set or type count is refused and
    leaves the destination unchanged."""
    from procell import _lib
    L = _lib.load()
    vals = [1.0, 2.5, 5.0]
    a, keep_a = _histogram(vals, [3, 0, 7], [[1, 2], [0, 0], [3, 4]], roots=5, divisions=9, leaves=10,
                           max_generation=4, sweeps=3, device_ms=1.5)
    b, keep_b = _histogram(vals, [2, 1, 2**40], [[2, 0], [1, 0], [2**39, 2**39]], roots=2, divisions=1, leaves=3,
                           max_generation=7, sweeps=2, device_ms=0.25)
    assert L.pc_histogram_accumulate(ctypes.byref(a), ctypes.byref(b)) == 0
    assert list(keep_a[1]) == [5, 1, 7 + 2**40]
    assert keep_a[2].tolist() == [[3, 2], [1, 0], [3 + 2**39, 4 + 2**39]]
    assert (a.stats.roots, a.stats.divisions, a.stats.leaves, a.stats.max_generation, a.stats.sweeps) == (7, 10, 13, 7, 5)
    assert a.stats.device_ms == 1.75
    before = keep_a[1].copy()
    c, keep_c = _histogram([1.0, 2.5, 5.000000001], [1, 1, 1], [[1, 0], [1, 0], [1, 0]])
    assert L.pc_histogram_accumulate(ctypes.byref(a), ctypes.byref(c)) == 1
    d, keep_d = _histogram(vals, [1, 1, 1], [[1], [1], [1]])
    assert L.pc_histogram_accumulate(ctypes.byref(a), ctypes.byref(d)) == 1
    assert np.array_equal(keep_a[1], before)
    assert L.pc_histogram_accumulate(None, ctypes.byref(a)) == 1
