"""Runs the reference binary on the small workload with many seeds and writes its output
histograms as a fixture. Run on a GPU machine from the repository root, after
`oracle/ref_build.sh` has built oracle/_ref/procell_ref:

    python tests/golden/make_reference_fixtures.py [--variant small|single_type] [--runs 64]

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

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "cuda-pro-cell_gb300"))

import procell.configs as cfg  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--runs", type=int, default=64)
    ap.add_argument("--variant", choices=["small", "single_type"], default="small",
                    help="single_type: the small histogram with one type (1.0, 48.33, 21.6)")
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    if a.out is None:
        a.out = os.path.join(HERE, f"reference_{a.variant}.json")
    ref = os.path.join(ROOT, "oracle", "_ref", "procell_ref")
    shim = os.path.join(ROOT, "oracle", "_ref", "libtimeshim.so")
    w = cfg.small()
    if a.variant == "single_type":
        w.types = [(1.0, 48.33, 21.6)]
    d = tempfile.mkdtemp()
    cfg.write_histogram(os.path.join(d, "h.txt"), w.bins)
    cfg.write_types(os.path.join(d, "c.txt"), w.types)
    runs = []
    for k in range(a.runs):
        stamp = 1764806400 + 7919 * k
        env = dict(os.environ, LD_PRELOAD=shim, PROCELL_REF_TIME=str(stamp))
        r = subprocess.run([ref, "-h", os.path.join(d, "h.txt"), "-c", os.path.join(d, "c.txt"),
                            "-t", repr(w.t_max), "-p", repr(w.phi)],
                           capture_output=True, text=True, env=env, timeout=600)
        if r.returncode != 0 or not r.stdout.strip():
            raise SystemExit(f"reference run {k} failed: rc={r.returncode} {r.stdout[-400:]} {r.stderr[-400:]}")
        rows = []
        for line in r.stdout.splitlines():
            v, c = line.split("\t")[:2]
            rows.append([float(v).hex(), int(c)])
        runs.append({"time": stamp, "rows": rows})
        print(f"run {k}: {sum(c for _, c in rows)} cells", flush=True)
    vals = sorted({v for r in runs for v, _ in r["rows"]}, key=float.fromhex)
    pos = {v: i for i, v in enumerate(vals)}
    counts = []
    for r in runs:
        c = [0] * len(vals)
        for v, n in r["rows"]:
            c[pos[v]] = n
        counts.append(c)
    out = {"workload": f"{a.variant} (procell.configs.small)", "types": w.types, "t_max": w.t_max, "phi": w.phi,
           "times": [r["time"] for r in runs], "values": vals, "counts": counts,
           "note": "values as float hex of the reference's %.10g text; counts[run][value]"}
    with open(a.out, "w") as fh:
        json.dump(out, fh, separators=(",", ":"))
    print("wrote", a.out)


if __name__ == "__main__":
    main()
