"""Measurement infrastructure: wall time of the reference binary against this engine's CLI.

Run on a GPU machine from the repository root, after `oracle/ref_build.sh` has built
oracle/_ref/procell_ref and `__graft_entry__.build()` this engine's CLI:

    python oracle/ref_timing.py [--runs 10] [--workload small|small_one_type|medium_t150] [--binary sm100|sm103a]

Both programs run as whole processes, the way a caller of the reference binary runs them:
CUDA initialisation, reading the two input files, the simulation and the histogram on
stdout. Workloads: the small one (procell.configs.small: 64 bins, about 1e4 initial cells,
t_max 168, phi the smallest value; with its two types or one), and the medium histogram and
types (1e6 initial cells, 4 types) with t_max 150, the largest configured input that the
reference's planner runs in one iteration (oracle/ref_planner.py: deepest generation 8
against a recursion depth of 9, grid and level sizes in range). Runs alternate between the
two binaries; the medians are reported. The reference is seeded through the preloaded time()
shim (oracle/_ref/libtimeshim.so), as in tests/golden/make_reference_fixtures.py. The
division count of this engine's run (the reference prints none) converts both wall times
into divisions per second of wall time. Prints one JSON line. The medium and large
workloads as configured are not run: the planner restatement shows they need a second
iteration, which reads uninitialised level slots as cells and computes its grid size in
uint16_t (src/simulation/proliferation.cu:245, :283).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "cuda-pro-cell_gb300"))

import procell.configs as cfg  # noqa: E402
from procell import _lib  # noqa: E402


def run(cmd, env=None):
    t = time.perf_counter()
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=600)
    dt = time.perf_counter() - t
    if r.returncode != 0 or not r.stdout.strip():
        raise SystemExit(f"{cmd[0]} failed: rc={r.returncode} {r.stdout[-300:]} {r.stderr[-300:]}")
    return dt, r.stdout


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--runs", type=int, default=10)
    ap.add_argument("--workload", choices=["small", "small_one_type", "medium_t150"], default="small")
    ap.add_argument("--binary", choices=["sm100", "sm103a"], default="sm100")
    a = ap.parse_args()
    ref = os.path.join(HERE, "_ref", "procell_ref_sm100" if a.binary == "sm100" else "procell_ref")
    shim = os.path.join(HERE, "_ref", "libtimeshim.so")
    ours = _lib.CLI_PATH
    w = cfg.small()
    if a.workload == "small_one_type":
        w.types = [(1.0, 48.33, 21.6)]
    elif a.workload == "medium_t150":
        w = cfg.medium()
        w.t_max = 150.0
    d = tempfile.mkdtemp()
    h, c = os.path.join(d, "h.txt"), os.path.join(d, "c.txt")
    cfg.write_histogram(h, w.bins)
    cfg.write_types(c, w.types)
    args = ["-h", h, "-c", c, "-t", repr(w.t_max), "-p", repr(w.phi)]
    t_ref, t_ours = [], []
    for k in range(a.runs + 1):  # run 0 of each is a warm-up (page cache, driver state)
        env = dict(os.environ, LD_PRELOAD=shim, PROCELL_REF_TIME=str(1764806400 + 7919 * k))
        dr, _ = run([ref] + args, env)
        do, _ = run([ours] + args + ["--seed", str(1000 + k)])
        if k:
            t_ref.append(dr)
            t_ours.append(do)
    from procell import Engine
    eng = Engine(0)
    divs = []
    for k in range(a.runs):
        divs.append(eng.simulate(w.bins, w.types, w.t_max, w.phi, 1000 + k).stats["divisions"])
    eng.close()
    div = statistics.median(divs)
    mr, mo = statistics.median(t_ref), statistics.median(t_ours)
    print(json.dumps({
        "workload": f"{a.workload} ({w.roots} initial cells, {len(w.types)} type(s), t_max {w.t_max})",
        "binary": os.path.basename(ref),
        "runs": a.runs,
        "reference_wall_s": {"median": mr, "min": min(t_ref), "max": max(t_ref)},
        "ours_wall_s": {"median": mo, "min": min(t_ours), "max": max(t_ours)},
        "divisions_per_run": div,
        "reference_divisions_per_wall_s": div / mr,
        "ours_divisions_per_wall_s": div / mo,
        "speedup": mr / mo,
    }))


if __name__ == "__main__":
    main()
