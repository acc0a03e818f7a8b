"""Run a named synthetic workload on the GPU and print its statistics.

    PYTHONPATH=cuda-pro-cell_gb300 python -m procell medium --runs 2 --budget 2e9

Workloads are those of procell.configs (small, medium, large, and batched: the first
--instances instances of the batched workload as one batch). --budget limits the device
memory of the level buffers (memory_budget_bytes), e.g. to keep a profiler capture small;
--driver and --config select the driver and the compiled sweep configuration; --t-max and
--phi replace the workload's (a larger phi makes the trees shallower, so a given budget
holds fewer, larger level buffers and each division sweep is longer); --root-end runs only
the first initial cells (a prefix of the same workload, e.g. for a small profiler capture).
"""
import argparse
import json
import time

from . import Engine
from . import configs


def main():
    ap = argparse.ArgumentParser(prog="python -m procell")
    ap.add_argument("workload", choices=["small", "medium", "large", "batched"])
    ap.add_argument("--instances", type=int, default=4096, help="batched: how many instances")
    ap.add_argument("--runs", type=int, default=1)
    ap.add_argument("--budget", type=float, default=0.0)
    ap.add_argument("--seed", type=int, default=None)
    ap.add_argument("--driver", type=int, default=0, help="0: one launch per sweep, 1: persistent")
    ap.add_argument("--config", type=int, default=4, help="compiled sweep configuration 0-7")
    ap.add_argument("--t-max", type=float, default=None)
    ap.add_argument("--phi", type=float, default=None)
    ap.add_argument("--root-end", type=int, default=None)
    a = ap.parse_args()
    if a.workload == "batched":
        return run_batched(a)
    w = configs.by_name(a.workload)
    if a.t_max is not None:
        w.t_max = a.t_max
    if a.phi is not None:
        w.phi = a.phi
    eng = Engine(0)
    if a.budget > 0:
        eng.set_option("memory_budget_bytes", a.budget)
    eng.set_option("driver", a.driver)
    eng.set_option("sweep_config", a.config)
    plan = eng.plan(w.bins, w.types, w.t_max, w.phi, w.seed if a.seed is None else a.seed)
    if a.root_end is not None:
        plan.set_roots(0, min(a.root_end, w.roots))
    for i in range(a.runs):
        t = time.perf_counter()
        plan.run()
        dt = time.perf_counter() - t
        s = plan.stats()
        print(json.dumps({"workload": a.workload, "run": i, "wall_ms": round(1e3 * dt, 3),
                          "divisions": s["divisions"], "sweeps": s["sweeps"],
                          "device_ms": round(s["device_ms"], 3)}), flush=True)
    plan.close()
    eng.close()


def run_batched(a):
    ws = configs.batched()[:a.instances]
    eng = Engine(0)
    if a.budget > 0:
        eng.set_option("memory_budget_bytes", a.budget)
    eng.set_option("driver", a.driver)
    eng.set_option("sweep_config", a.config)
    b = eng.batch([(w.bins, w.types, w.t_max, w.phi, w.seed) for w in ws])
    for i in range(a.runs):
        t = time.perf_counter()
        b.run()
        dt = time.perf_counter() - t
        s = b.stats()
        print(json.dumps({"workload": "batched", "instances": len(ws), "run": i, "wall_ms": round(1e3 * dt, 3),
                          "divisions": s["divisions"], "sweeps": s["sweeps"],
                          "device_ms": round(s["device_ms"], 3)}), flush=True)
    b.close()
    eng.close()


if __name__ == "__main__":
    main()
