"""Runs the reference binary on a workload with many seeds and writes its output histograms
as a fixture. Run on a GPU machine from the repository root, after `oracle/ref_build.sh` has
built oracle/_ref/procell_ref (sm_103a) and oracle/_ref/procell_ref_sm100 (sm_100):

    python tests/golden/make_reference_fixtures.py [--variant V] [--runs 64] [--binary sm100|sm103a]

Variants (procell.configs.small's histogram unless stated):
  small        the configured two types (0.53, 48.33, 21.6), (0.47, 86.3, 26.8);
  single_type  one type (1.0, 48.33, 21.6);
  same_timer   two types that share (mean, sd) = (48.33, 21.6), ratios 0.53 / 0.47, run with
               -r so each run also records the per-type columns: the type drawn cannot change
               the totals, only which column a leaf is counted in;
  medium_t150  the medium workload's histogram and types (1e6 initial cells) with t_max 150,
               the largest input the reference's planner runs in one iteration
               (oracle/ref_planner.py); 16 runs by default, wall time of each recorded;
  medium_t150_same_timer  the same histogram and t_max with three types that share
               (mean, sd) = (60, 18), ratios 0.4 / 0.35 / 0.25, no quiescent type: the type
               drawn cannot change the totals, so any loss of cells (a child grid the
               reference failed to launch) or any extra cell would show in them.

The reference seeds every random stream with time(NULL); the preloaded oracle/_ref
libtimeshim.so returns PROCELL_REF_TIME instead, so the runs are reproducible. Run k gets the
timestamp 1764806400 + 7919 k: realistic values matter, because the reference derives the
second daughter's seed as `seed - timer * 1e4 + id` in double arithmetic
(src/simulation/proliferation.cu:331), which would turn negative (and saturate when converted
to uint64) for a small time value. Each run is checked for a zero exit status and a non-empty histogram.
The fixture (tests/golden/reference_<variant>.json) holds the output values (float hex of
the printed text) and, per run, the count of each; the CPU suite compares their
distribution with the oracle's.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "cuda-pro-cell_gb300"))

import procell.configs as cfg  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--runs", type=int, default=64)
    ap.add_argument("--variant", choices=["small", "single_type", "same_timer", "medium_t150", "medium_t150_same_timer"],
                    default="small")
    ap.add_argument("--binary", choices=["sm100", "sm103a"], default="sm100")
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    if a.out is None:
        a.out = os.path.join(HERE, f"reference_{a.variant}.json")
    ref = os.path.join(ROOT, "oracle", "_ref", "procell_ref_sm100" if a.binary == "sm100" else "procell_ref")
    shim = os.path.join(ROOT, "oracle", "_ref", "libtimeshim.so")
    w = cfg.small()
    track = False
    source = "procell.configs.small"
    if a.variant == "single_type":
        w.types = [(1.0, 48.33, 21.6)]
    elif a.variant == "same_timer":
        w.types = [(0.53, 48.33, 21.6), (0.47, 48.33, 21.6)]
        track = True
    elif a.variant in ("medium_t150", "medium_t150_same_timer"):
        w = cfg.medium()
        w.t_max = 150.0
        source = "procell.configs.medium, t_max 150"
        if a.variant == "medium_t150_same_timer":
            w.types = [(0.4, 60.0, 18.0), (0.35, 60.0, 18.0), (0.25, 60.0, 18.0)]
            source += ", three types sharing (60, 18)"
    d = tempfile.mkdtemp()
    cfg.write_histogram(os.path.join(d, "h.txt"), w.bins)
    cfg.write_types(os.path.join(d, "c.txt"), w.types)
    runs = []
    for k in range(a.runs):
        stamp = 1764806400 + 7919 * k
        env = dict(os.environ, LD_PRELOAD=shim, PROCELL_REF_TIME=str(stamp))
        t0 = time.perf_counter()
        r = subprocess.run([ref, "-h", os.path.join(d, "h.txt"), "-c", os.path.join(d, "c.txt"),
                            "-t", repr(w.t_max), "-p", repr(w.phi)] + (["-r"] if track else []),
                           capture_output=True, text=True, env=env, timeout=600)
        wall = time.perf_counter() - t0
        if r.returncode != 0 or not r.stdout.strip():
            raise SystemExit(f"reference run {k} failed: rc={r.returncode} {r.stdout[-400:]} {r.stderr[-400:]}")
        rows = []
        for line in r.stdout.splitlines():
            f = line.split("\t")
            rows.append([float(f[0]).hex(), int(f[1])] + [int(x) for x in f[2:]])
        runs.append({"time": stamp, "rows": rows, "wall": wall})
        print(f"run {k}: {sum(x[1] for x in rows)} cells, {wall:.3f} s", flush=True)
    vals = sorted({x[0] for r in runs for x in r["rows"]}, key=float.fromhex)
    pos = {v: i for i, v in enumerate(vals)}
    counts, per_type = [], []
    for r in runs:
        c = [0] * len(vals)
        pt = [[0] * len(w.types) for _ in vals]
        for x in r["rows"]:
            c[pos[x[0]]] = x[1]
            if track:
                pt[pos[x[0]]] = x[2:]
        counts.append(c)
        per_type.append(pt)
    out = {"workload": f"{a.variant} ({source})", "binary": os.path.basename(ref), "types": w.types,
           "t_max": w.t_max, "phi": w.phi, "times": [r["time"] for r in runs],
           "wall_s": [round(r["wall"], 4) for r in runs], "values": vals, "counts": counts,
           "note": "values as float hex of the reference's %.10g text; counts[run][value]"
                   + ("; per_type[run][value][type], types in file order (-r)" if track else "")}
    if track:
        out["per_type"] = per_type
    with open(a.out, "w") as fh:
        json.dump(out, fh, separators=(",", ":"))
    print("wrote", a.out)


if __name__ == "__main__":
    main()
