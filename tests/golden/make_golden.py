"""Regenerates tests/golden/*.json from the CPU oracle (run from the repository root):

    python tests/golden/make_golden.py

The reference ships no tests or golden data (and seeds every run with time(NULL)), so these
fixtures record the oracle's outputs on fixed inputs and seeds: the Philox4x32-10 blocks of
a few counters, the first normals of a node range, the ziggurat tables, and full output
histograms of the small workload and of edge cases. The CPU suite checks the oracle still
produces them; the GPU suite checks the engine does.
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "cuda-pro-cell_gb300"))

import numpy as np  # noqa: E402

import oracle  # noqa: E402
import procell.configs as cfg  # noqa: E402

CASES = {
    "small_seed11": (lambda w: dict(bins=w.bins, types=w.types, t_max=w.t_max, phi=w.phi, seed=w.seed))(cfg.small()),
    "small_seed7": (lambda w: dict(bins=w.bins, types=w.types, t_max=w.t_max, phi=w.phi, seed=7))(cfg.small()),
    "readme_example": dict(bins=[(1.0, 0), (8.144, 53), (9823.85, 274)],
                           types=[(0.53, 48.33, 21.6), (0.29, 86.3, 26.8), (0.18, -1.0, -1.0)],
                           t_max=120.0, phi=None, seed=2024),
    "quiescent_and_zero_mean": dict(bins=[(64.0, 40), (10.0, 5), (0.75, 3)],
                                    types=[(0.4, 0.0, 1.0), (0.35, 5.0, 1.0), (0.25, -1.0, -1.0)],
                                    t_max=30.0, phi=1.0, seed=5),
    "heavy_truncation": dict(bins=[(4096.0, 300)], types=[(1.0, 1.0, 3.0)], t_max=12.0, phi=1.0, seed=3),
}


def tables_digest():
    k, w, f = oracle.tables()
    h = hashlib.sha256()
    for a in (k, w.view(np.uint32), f.view(np.uint32)):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def main():
    rng = np.random.default_rng(99)
    ctrs = rng.integers(0, 2 ** 32, size=(16, 4), dtype=np.uint64).astype(int).tolist()
    key = [0x12345678, 0x9ABCDEF0]
    philox = [{"ctr": c, "key": key, "out": oracle.philox(c, key)} for c in ctrs]
    z = oracle.normals(seed=77, root=5, first_parent=1000, count=256)
    out = {"philox": philox,
           "normals": {"seed": 77, "root": 5, "first_parent": 1000,
                       "bits": [int(x) for x in z.view(np.uint32)]},
           "tables_sha256": tables_digest(),
           "cases": {}}
    for name, c in CASES.items():
        r = oracle.simulate(c["bins"], c["types"], c["t_max"], c["phi"], seed=c["seed"])
        nz = [i for i in range(len(r.values)) if int(r.totals[i])]
        out["cases"][name] = {
            "input": {"bins": [[float(v), int(f)] for v, f in c["bins"]], "types": [list(t) for t in c["types"]],
                      "t_max": c["t_max"], "phi": c["phi"], "seed": c["seed"]},
            "values": [float(r.values[i]).hex() for i in nz],
            "per_type": [[int(x) for x in r.per_type[i]] for i in nz],
            "stats": r.stats,
            "text": oracle.format_histogram(r, True),
        }
    with open(os.path.join(HERE, "oracle_golden.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
        fh.write("\n")
    print("wrote", os.path.join(HERE, "oracle_golden.json"))


if __name__ == "__main__":
    main()
