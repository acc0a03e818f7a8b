#!/usr/bin/env python3
"""Benchmark of the proliferation path: cell divisions/s, instances/s, fwd+bwd grads/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload large|medium|small]
    python bench.py --workload batched|calibration     # one of the other forms alone
    python bench.py --impl reference ...               # the CPU arm (see below)

One step = one complete simulation of the workload (root sweep + every division sweep)
from inputs already resident in HBM (`value`), and the same through the C ABI with host
buffers, the upload and the histogram download inside the timed region (`e2e`). The
default workload is the 1e7-cell configuration: 4096 bins, fluorescence log-uniform on
[1, 1e6], Poisson(2500) cells per bin, five types (means U[30, 60], sd 0.3 x mean,
Dirichlet ratios), t_max 336, phi 1; 3.55e9 divisions per step.

On one GPU the default line also carries, under "forms", the two other metrics of the path,
each measured with its own value, e2e, roofline, CPU baseline and clocks: "batched" (4096
uneven instances in one run, instances/s, against looping the plain form, every instance
checked bit for bit against its plain run) and "calibration" (forward + loss gradient +
adjoint of the smoothed form for 256 candidates, grads/s; Levenberg-Marquardt on the
smoothed form against particle swarms to equal loss on five inputs, scored on the accurate
smoothed loss and on the plain simulator's loss averaged over 16 seeds). --no-forms skips
them.

Under torchrun each rank runs its own instance (seed + rank) of the workload on its own
GPU: weak scaling, no collective on the data path; value = all ranks' divisions / the
slowest rank's time.

The reference has no CPU implementation of this path (every step of it is a CUDA kernel),
so `--impl reference` times the CPU restatement of the reference's algorithm (the oracle)
on all host cores, over a bounded sample of the same workload's initial cells.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "cuda-pro-cell_gb300")
sys.path.insert(0, PKG)

METRIC = "cell divisions/s"
UNIT = "divisions/s"
ALG_BYTES_PER_NODE = 32  # 16-byte cell state written once and read once per tree node
FP64_OPS_PER_DIVISION = 4  # per daughter: tau = fma(sd, z, mean) and due = birth + tau


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples (200 ms) while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        top = max(sm)
        loaded = [s for s in sm if s >= 0.5 * top] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(name):
    import procell.configs as cfg
    return cfg.by_name(name)


def describe(w):
    return (f"{w.name}: {len(w.bins)} bins, {w.roots} initial cells, {len(w.types)} types, "
            f"t_max {w.t_max:g}, phi {w.phi:g}")


def cpu_sample(w, target_s, nthreads, oracle):
    """Oracle divisions/s on a prefix of the workload's initial cells sized to ~target_s:
    a probe run sizes the sample, which grows (at most three times) while it runs under half
    the target."""
    n = w.roots
    m = max(1, n // 2048)
    for _ in range(4):
        t = time.perf_counter()
        r = oracle.simulate(w.bins, w.types, w.t_max, w.phi, seed=w.seed, root_end=m, nthreads=nthreads)
        dt = max(time.perf_counter() - t, 1e-3)
        if dt >= 0.5 * target_s or m >= n:
            break
        m = int(min(n, max(m + 1, m * target_s / dt)))
    return r.stats["divisions"], dt, m


def cpu_model():
    """The host CPU as /proc/cpuinfo or lscpu names it (for the record)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.split(":")[0].strip() in ("Model name", "Model Name"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as fh:
            for ln in fh:
                if ln.lower().startswith("model name"):
                    return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    if args.workload == "batched":
        return run_reference_batched(args)
    if args.workload == "calibration":
        return run_reference_calibration(args)
    w = workload(args.workload)
    cores = os.cpu_count() or 1
    per_step = max(2.0, args.cpu_seconds / 2)
    for _ in range(args.warmup):
        cpu_sample(w, per_step / 4, cores, oracle)
    divs, secs, samples = 0, 0.0, []
    for _ in range(args.steps):
        d, s, m = cpu_sample(w, per_step, cores, oracle)
        divs += d
        secs += s
        samples.append(m)
    value = divs / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generator, procell/configs.py)",
        "config": {"workload": describe(w), "sample": "first %d of %d initial cells per step" % (min(samples), w.roots)},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "oracle (CPU restatement of the reference algorithm) on the first "
                                   "%d-%d of %d initial cells per step, %d threads"
                                   % (min(samples), max(samples), w.roots, cores),
                         "cpu_model": cpu_model()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if not args.no_forms:
        # the CPU restatements of the other two forms, one bounded sample each
        cs = max(4.0, args.cpu_seconds / 2)
        line["forms"] = {"batched": reference_batched_line(1, 0, cs),
                         "calibration": reference_calibration_line(1, 0, cs)}
    print(json.dumps(line), flush=True)
    return 0


def run_reference_batched(args):
    print(json.dumps(reference_batched_line(args.steps, args.warmup, max(2.0, args.cpu_seconds / 2))), flush=True)
    return 0


def reference_batched_line(steps, warmup, per_step):
    instances = batched_instances()
    for _ in range(warmup):
        cpu_batched_sample(instances, per_step / 4)
    vals, secs = [], 0.0
    for _ in range(steps):
        c = cpu_batched_sample(instances, per_step)
        vals.append(c)
    done = sum(float(c["sample"].split()[2]) for c in vals)
    secs = sum(float(c["sample"].split("(")[1].split()[0]) for c in vals)
    value = done / secs
    line = {
        "impl": "reference", "metric": "instances/s (batched form)", "value": value, "unit": "instances/s",
        "n_gpus": 1, "steps": steps, "warmup": warmup, "ms_per_step": 1e3 * secs / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generator, procell/configs.py batched())",
        "config": {"workload": "batched: %d instances" % len(instances),
                   "sample": "instances drawn at random, about %.0f s per step" % per_step},
        "cpu_baseline": {"value": value, "unit": "instances/s", "cores": vals[0]["cores"], "kind": "port",
                         "sample": "; ".join(c["sample"] for c in vals)},
        "e2e": {"value": value, "unit": "instances/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    return line


def run_ours(args):
    import numpy as np
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    if rank == 0:
        import build as pkg_build
        pkg_build.build()
    if world > 1:
        torch.distributed.barrier()
    from procell import Engine

    w = workload(args.workload)
    roots_split = args.split == "roots"
    seed = w.seed if roots_split else w.seed + rank
    eng = Engine(local)
    stream = torch.cuda.current_stream()
    eng.set_stream(stream.cuda_stream)
    plan = eng.plan(w.bins, w.types, w.t_max, w.phi, seed)
    shard = None
    if roots_split:
        # one input split over the ranks: a contiguous range of initial cells per rank,
        # balanced by expected work, and one sum of the counts per step
        from procell.distributed import shard_range_weighted
        shard = shard_range_weighted(w.bins, w.types, w.t_max, w.phi, rank, world)
        plan.set_roots(*shard)
    tuning = eng.autotune(plan, repeats=1) if not args.no_tune else None

    def reduce_counts():
        # the sharded step's one exchange: an element-wise sum of the (generation, bin, type)
        # counts over the ranks
        if roots_split and world > 1:
            t = torch.from_numpy(plan.raw_counts().view(np.int64)).to("cuda")
            torch.distributed.all_reduce(t)
            return t
        return None

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        plan.run()
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    divisions = roots = sweeps = kernels = 0
    divide_ms = device_ms = 0.0
    e0.record(stream)
    for _ in range(args.steps):
        plan.run()
        reduce_counts()
        st = plan.stats()
        divisions += st["divisions"]
        roots += st["roots"]
        sweeps += st["sweeps"]
        kernels += st["kernel_launches"]
        divide_ms += st["divide_ms"]
        device_ms += st["device_ms"]
    e1.record(stream)
    barrier()
    elapsed_ms = e0.elapsed_time(e1)

    # end to end through the C ABI: host inputs (the histogram as a pc_bin array in host
    # memory, as pc_load_histogram returns it), upload, run, histogram download + merge
    from procell import _lib
    bins_host = _lib.bins_numpy(w.bins)
    e2e_t = 0.0
    h2d = d2h = 0
    e2e_div = 0
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        if roots_split:
            res = eng.simulate(bins_host, w.types, w.t_max, w.phi, seed, root_begin=shard[0], root_end=shard[1])
            if world > 1:
                tot = torch.from_numpy(res.per_type.view(np.int64)).to("cuda")
                torch.distributed.all_reduce(tot)
                tot.cpu()
        else:
            res = eng.simulate(bins_host, w.types, w.t_max, w.phi, seed)
        if i < args.warmup:  # untimed: the context's first merge scratch and spare buffers
            continue
        e2e_t += time.perf_counter() - t
        h2d += res.stats["h2d_bytes"]
        d2h += res.stats["d2h_bytes"]
        e2e_div += res.stats["divisions"]
    clk = clocks.stop()
    barrier()

    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([elapsed_ms, e2e_t], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        s = torch.tensor([divisions, e2e_div], dtype=torch.float64, device="cuda")
        dist.all_reduce(s, op=dist.ReduceOp.SUM)
        elapsed_ms, e2e_t = float(t[0]), float(t[1])
        tot_div, tot_e2e_div = float(s[0]), float(s[1])
    else:
        tot_div, tot_e2e_div = float(divisions), float(e2e_div)
    if rank != 0:
        return 0

    hbm, peak_kind = peaks()
    # dominant kernel: the division sweep. Algorithmic bytes: each division creates two
    # tree nodes, each node's 16-byte state written once and read once (32 B per node).
    alg_bytes = 2 * ALG_BYTES_PER_NODE * divisions
    persistent = bool(tuning and tuning["driver"])
    launches = max(1, args.steps if persistent else sweeps)  # launches of the dominant kernel
    achieved = alg_bytes / (divide_ms * 1e-3) / 1e9 if divide_ms > 0 else None
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic_per_division_persistent.txt" if persistent
                         else "traffic_per_division.txt")
    if os.path.exists(tpath):
        try:
            per_div = float(open(tpath).read().split()[0])
            traffic = per_div * divisions / launches
        except (ValueError, IndexError):
            traffic = None
    # the division sweep's other ceilings: the FP64 pipe (two FMA + two adds per division,
    # the daughters' exact due times) against its measured peak, and instruction issue
    # (warp instructions per division from the ncu summary in profiles/) against four
    # issue slots per SM per cycle at the sampled SM clock
    fp64_peak = eng.peak("fp64")
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    ipd = None
    try:
        with open(os.path.join(ROOT, "profiles", "instructions_per_division.txt")) as fh:
            ipd = float(fh.read().split()[0])
    except (OSError, ValueError, IndexError):
        pass
    fp64_rate = FP64_OPS_PER_DIVISION * divisions / (divide_ms * 1e-3) if divide_ms > 0 else None
    issue_frac = None
    if ipd and divide_ms > 0 and clk.get("sm_mhz"):
        issue_frac = ipd * divisions / (divide_ms * 1e-3) / (4.0 * sms * clk["sm_mhz"] * 1e6)
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        oracle.build()
        cores = os.cpu_count() or 1
        d, s, m = cpu_sample(w, args.cpu_seconds, cores, oracle)
        d1, s1, m1 = cpu_sample(w, max(2.0, args.cpu_seconds / 3), 1, oracle)
        cpu = {"value": d / s, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": "oracle on the first %d of %d initial cells (%.1f s, %d divisions)"
                         % (m, w.roots, s, d),
               "single_thread": {"value": d1 / s1, "sample": "first %d initial cells, %.1f s" % (m1, s1)},
               "cpu_model": cpu_model(), "nproc": cores}
    line = {
        "metric": METRIC,
        "value": tot_div / (elapsed_ms * 1e-3),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": elapsed_ms / args.steps,
        "higher_is_better": True,
        "scaling": "strong" if roots_split else "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded generator, procell/configs.py)",
        "config": {"workload": describe(w), "divisions_per_step": divisions // args.steps,
                   "nodes_per_step": (roots + 2 * divisions) // args.steps,
                   "l2": "no flush: each step streams %.0f GB of level buffers, >> 129 MB L2"
                         % (2 * 16 * divisions / args.steps / 1e9),
                   "parallelism": (f"one input, initial cells split over {world} GPUs by expected work, "
                                   f"one all_reduce of the counts per step" if roots_split
                                   else f"one independent instance per GPU x{world}"),
                   "tuning": tuning},
        "e2e": {"value": tot_e2e_div / e2e_t, "unit": UNIT,
                "h2d_bytes_per_step": h2d // args.steps, "d2h_bytes_per_step": d2h // args.steps},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": (achieved / hbm) if achieved else None, "traffic": traffic,
                     "peak_source": peak_kind,
                     "dram_achieved": (traffic * launches / (divide_ms * 1e-3) / 1e9)
                     if (traffic and divide_ms > 0) else None,
                     "dram_frac": (traffic * launches / (divide_ms * 1e-3) / 1e9 / hbm)
                     if (traffic and divide_ms > 0) else None,
                     "kernel": "k_persist" if (tuning and tuning["driver"]) else "k_divide",
                     "launches_per_step": launches / args.steps,
                     "alg_bytes_per_launch": alg_bytes / launches,
                     "fp64_achieved": fp64_rate, "fp64_peak": fp64_peak,
                     "fp64_frac": (fp64_rate / fp64_peak) if (fp64_rate and fp64_peak) else None,
                     "fp64_unit": "FP64 lane-ops/s (%d per division; peak: pc_debug_peak FMA probe)"
                                  % FP64_OPS_PER_DIVISION,
                     "issue_frac": issue_frac,
                     "issue_note": "%s warp instructions per division (ncu, profiles/) x divisions / "
                                   "(4 x %d SMs x sampled SM clock)" % (ipd, sms),
                     "note": "alg bytes = 64 B per division (two 16-B nodes written+read); the "
                             "kernel stores only daughters that divide again, so its DRAM traffic "
                             "(dram_achieved, from the ncu bytes per division in profiles/) is about "
                             "half of that and the sweep is bound by instruction issue, not HBM"
                             + ("; the persistent launch also runs the root sweep" if persistent else "")},
        "gpu_launches": kernels,
        "clocks": clk,
        "device_ms_per_step": device_ms / args.steps,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    if world == 1 and not args.no_forms:
        # the other two metrics of the path, each with its own value, e2e, roofline, CPU
        # baseline and clocks: the batched form and the smoothed form's calibration
        plan.close()
        cs = None if args.no_cpu_baseline else max(4.0, args.cpu_seconds / 2)
        line["forms"] = {
            "batched": measure_batched(eng, local, args.steps, args.warmup, not args.no_tune, cs,
                                       min(args.steps, 5)),
            "calibration": measure_calibration(eng, local, args.steps, args.warmup, cs, pso_seconds=15.0,
                                               extra_seeds=(8, 9, 10, 11), extra_pso_seconds=8.0),
        }
    print(json.dumps(line), flush=True)
    return 0


def batched_instances():
    """The batched workload as (bins, types, t_max, phi, seed) rows with numpy bins."""
    import numpy as np
    import procell.configs as cfg
    out = []
    for w in cfg.batched():
        v = np.array([b[0] for b in w.bins], np.float64)
        f = np.array([b[1] for b in w.bins], np.uint64)
        out.append(((v, f), w.types, w.t_max, w.phi, w.seed))
    return out


def simulate_batch_e2e(eng, instances):
    """pc_simulate_batch with host inputs: upload, run, every instance's merged histogram
    back on the host. Returns (seconds, h2d bytes, d2h bytes, divisions)."""
    import ctypes
    from procell import _lib
    keep = []
    arr = (_lib.Instance * len(instances))()
    for i, (bins, types, t_max, phi, seed) in enumerate(instances):
        b, t = _lib.bins_numpy(bins), _lib.types_numpy(types)
        keep += [b, t]
        arr[i].bins = b.ctypes.data_as(ctypes.POINTER(_lib.Bin))
        arr[i].n_bins = len(b)
        arr[i].types = t.ctypes.data_as(ctypes.POINTER(_lib.CellType))
        arr[i].n_types = len(t)
        arr[i].t_max, arr[i].phi, arr[i].seed = t_max, phi, seed
    hs = (_lib.Histogram * len(instances))()
    t0 = time.perf_counter()
    rc = eng.L.pc_simulate_batch(eng.ctx, arr, len(instances), hs)
    dt = time.perf_counter() - t0
    eng._check(rc)
    h2d = sum(len(k) * k.itemsize for k in keep)
    d2h = sum(int(h.n_values) * 8 * (2 + int(h.n_types)) for h in hs)
    for h in hs:
        eng.L.pc_histogram_free(ctypes.byref(h))
    return dt, h2d, d2h


def run_batched(args):
    """Batched form alone: instances/s of one batch run against looping the plain form."""
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if rank != 0 and world > 1:
        return 0  # one GPU: the batched workload is a single-GPU job
    import build as pkg_build
    pkg_build.build()
    from procell import Engine
    eng = Engine(local)
    line = measure_batched(eng, local, args.steps, args.warmup, not args.no_tune,
                           None if args.no_cpu_baseline else args.cpu_seconds, args.steps)
    print(json.dumps(line), flush=True)
    return 0


def measure_batched(eng, local, steps, warmup, tune, cpu_seconds, e2e_steps):
    """The batched workload's line: `steps` timed batch runs from HBM-resident inputs,
    `e2e_steps` pc_simulate_batch calls with host inputs and outputs, one loop of the plain
    form over the same instances, per-instance parity against that loop, and (cpu_seconds
    not None) the oracle's instances/s on a sample of the instances."""
    import numpy as np
    import torch

    instances = batched_instances()
    n = len(instances)
    stream = torch.cuda.current_stream()
    eng.set_stream(stream.cuda_stream)
    batch = eng.batch(instances)
    tuning = eng.autotune(batch, repeats=1) if tune else None
    for _ in range(warmup):
        batch.run()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    divisions = roots = sweeps = kernels = 0
    divide_ms = device_ms = 0.0
    e0.record(stream)
    for _ in range(steps):
        batch.run()
        st = batch.stats()
        divisions += st["divisions"]
        roots += st["roots"]
        sweeps += st["sweeps"]
        kernels += st["kernel_launches"]
        divide_ms += st["divide_ms"]
        device_ms += st["device_ms"]
    e1.record(stream)
    torch.cuda.synchronize()
    elapsed_ms = e0.elapsed_time(e1)
    # the same batch as one persistent cooperative launch per run, replayed from a CUDA graph
    # (the autotuner keeps whichever driver is faster; both are reported)
    cfg_sel = tuning["config"] if tuning else 4
    eng.set_option("sweep_config", cfg_sel)
    eng.set_option("driver", 1)
    eng.set_option("graph", 1)
    for _ in range(2):
        batch.run()
    torch.cuda.synchronize()
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    for _ in range(steps):
        batch.run()
    g1.record(stream)
    torch.cuda.synchronize()
    graph_ms = g0.elapsed_time(g1) / steps
    graph_div = batch.stats()["divisions"]
    eng.set_option("driver", tuning["driver"] if tuning else 0)
    eng.set_option("graph", tuning["driver"] if tuning else 0)
    e2e_t = h2d = d2h = 0
    for k in range(1 + e2e_steps):
        dt, hb, db = simulate_batch_e2e(eng, instances)
        if k == 0:  # untimed: the context's first pinned stages and spare buffers
            continue
        e2e_t += dt
        h2d += hb
        d2h += db
    clk = clocks.stop()
    batch_counts = [batch.raw_counts(i) for i in range(n)]
    batch.close()

    # Looping the plain form over the same instances, with the same tuned configuration:
    # (a) one pc_simulate per instance (host inputs in, merged histogram out), against e2e;
    # (b) plans created beforehand, one pc_plan_run per instance, against value; the same
    #     plans give the per-instance parity check.
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for bins, types, t_max, phi, seed in instances:
        eng.simulate(bins, types, t_max, phi, seed)
    torch.cuda.synchronize()
    loop_e2e_s = time.perf_counter() - t0
    plans = [eng.plan(*x) for x in instances]
    for p in plans[:64]:
        p.run()
    torch.cuda.synchronize()
    t_each = np.zeros(n)
    t0 = time.perf_counter()
    for i, p in enumerate(plans):
        ti = time.perf_counter()
        p.run()  # returns when the run has finished
        t_each[i] = time.perf_counter() - ti
    torch.cuda.synchronize()
    loop_run_s = time.perf_counter() - t0
    d_each = np.array([p.stats()["divisions"] for p in plans], np.float64)
    same = sum(int(np.array_equal(p.raw_counts(), batch_counts[i])) for i, p in enumerate(plans))
    # the loop's time split: t_i = overhead + divisions_i x cost per division (least squares);
    # an instance is overhead-bound when the fixed part is the larger
    A = np.stack([np.ones(n), d_each], axis=1)
    (ovh, per_div), *_ = np.linalg.lstsq(A, t_each, rcond=None)
    ob = ovh > per_div * d_each
    split = {"overhead_ms_per_instance": 1e3 * ovh, "ns_per_division": 1e9 * per_div,
             "overhead_bound_instances": int(ob.sum()),
             "overhead_bound_time_share": float(t_each[ob].sum() / t_each.sum()),
             "overhead_time_share": float(n * ovh / t_each.sum()),
             "speedup_bound_at_plain_cost": float(t_each.sum() / max(1e-12, t_each.sum() - n * ovh)),
             "what": "plain runs timed one by one, t_i = overhead + divisions_i x cost (least squares); "
                     "overhead-bound: the fixed part is the larger; a batch removes the overhead only, so at "
                     "the plain per-division cost its speedup is at most loop time / (loop time - n x overhead)"}
    for p in plans:
        p.close()

    hbm, peak_kind = peaks()
    alg_bytes = 2 * ALG_BYTES_PER_NODE * divisions
    persistent = bool(tuning and tuning["driver"])
    launches = max(1, steps if persistent else sweeps)
    achieved = alg_bytes / (divide_ms * 1e-3) / 1e9 if divide_ms > 0 else None
    value = n * steps / (elapsed_ms * 1e-3)
    e2e_value = n * e2e_steps / e2e_t
    cpu = None
    if cpu_seconds:
        cpu = cpu_batched_sample(instances, cpu_seconds)
    line = {
        "metric": "instances/s (batched form)",
        "value": value,
        "unit": "instances/s",
        "n_gpus": 1,
        "steps": steps,
        "warmup": warmup,
        "ms_per_step": elapsed_ms / steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded generator, procell/configs.py batched())",
        "config": {"workload": "batched: %d instances, %d initial cells, bins U[32,1024], cells "
                               "log-U[1e3,1e6], 1-4 types (+quiescent 20%%), t_max U[48,336], "
                               "fluorescence log-U[1,1e4], phi = min nonzero bin" % (n, roots // steps),
                   "divisions_per_step": divisions // steps,
                   "nodes_per_step": (roots + 2 * divisions) // steps,
                   "tuning": tuning,
                   "l2": "no flush: each step streams %.0f GB of level buffers, >> 129 MB L2"
                         % (2 * 16 * divisions / steps / 1e9)},
        "divisions_per_s": divisions / (elapsed_ms * 1e-3),
        "loop_plain": {"run_instances_per_s": n / loop_run_s,
                       "e2e_instances_per_s": n / loop_e2e_s,
                       "run": "plans created beforehand, one pc_plan_run per instance",
                       "e2e": "one pc_simulate per instance (host inputs, merged histogram out)"},
        "speedup_vs_loop_plain": value / (n / loop_run_s),
        "persistent_graph": {"ms_per_step": graph_ms, "instances_per_s": n / (graph_ms * 1e-3),
                             "divisions_per_s": graph_div / (graph_ms * 1e-3), "launches_per_step": 1,
                             "speedup_vs_loop_plain": (n / (graph_ms * 1e-3)) / (n / loop_run_s),
                             "what": "the batch as one persistent cooperative launch per run, replayed from a "
                                     "CUDA graph, configuration %d" % cfg_sel},
        "loop_split": split,
        "e2e_speedup_vs_loop_plain": e2e_value / (n / loop_e2e_s),
        "bit_exact_instances": "%d/%d" % (same, n),
        "e2e": {"value": e2e_value, "unit": "instances/s", "h2d_bytes_per_step": h2d // e2e_steps,
                "d2h_bytes_per_step": d2h // e2e_steps, "steps": e2e_steps},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": (achieved / hbm) if achieved else None, "traffic": batched_traffic(divisions, launches),
                     "peak_source": peak_kind, "kernel": "k_persist" if persistent else "k_divide",
                     "launches_per_step": launches / steps,
                     "alg_bytes_per_launch": alg_bytes / launches},
        "gpu_launches": kernels,
        "clocks": clk,
        "device_ms_per_step": device_ms / steps,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    return line


def cpu_smooth_sample(bins, phi, t_max, h, paths, seed, params, seconds):
    """Candidate-gradients/s of the CPU restatement of the smoothed form (oracle_smooth: C++,
    FP64, all host cores) on one candidate: the forward pass, the loss gradient, the adjoint
    pass, over a prefix of the bins sized to ~`seconds`, scaled to the whole input by its share
    of initial cells."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    cores = os.cpu_count() or 1
    P = np.asarray(params, dtype=np.float64).reshape(1, -1, 3)
    total = sum(f for _, f in bins)
    nb, spent, cells = 1, 0.0, 0
    while True:
        sub = bins[:nb]
        cells = sum(f for _, f in sub)
        t = time.perf_counter()
        E, _ = oracle.smooth(sub, t_max, phi, h, paths, seed, P, nthreads=cores)
        oracle.smooth(sub, t_max, phi, h, paths, seed, P, np.ones_like(E), nthreads=cores)
        spent = time.perf_counter() - t
        if spent >= 0.4 * seconds or nb >= len(bins):
            break
        nb = min(len(bins), max(nb + 1, int(nb * 0.5 * seconds / max(spent, 1e-3))))
    reps = 1
    if nb >= len(bins) and spent < 0.4 * seconds:
        # the whole input is quick: repeat it for a steadier figure
        reps = max(1, int(0.4 * seconds / max(spent, 1e-3)))
        t = time.perf_counter()
        for _ in range(reps):
            E, _ = oracle.smooth(bins, t_max, phi, h, paths, seed, P, nthreads=cores)
            oracle.smooth(bins, t_max, phi, h, paths, seed, P, np.ones_like(E), nthreads=cores)
        spent = (time.perf_counter() - t) / reps
    per_grad = spent * total / max(1, cells)
    return {"value": 1.0 / per_grad, "unit": "grads/s", "cores": cores, "kind": "port",
            "sample": "oracle_smooth (C++ restatement of the smoothed form, FP64, %d threads) forward + "
                      "backward of one candidate on the first %d of %d bins (%d of %d initial cells, %.3f s "
                      "per pass pair, %d repetitions), scaled by initial cells"
                      % (cores, nb, len(bins), cells, total, spent, reps)}


def run_reference_calibration(args):
    print(json.dumps(reference_calibration_line(args.steps, args.warmup, max(2.0, args.cpu_seconds / 2))),
          flush=True)
    return 0


def reference_calibration_line(steps, warmup, per_step):
    from procell import calibrate as cb
    bins, phi, hidden = cb.problem_inputs(7)
    for _ in range(warmup):
        cpu_smooth_sample(bins, phi, 168.0, 0.5, 2, 7 + 2000, hidden, per_step / 4)
    vals = [cpu_smooth_sample(bins, phi, 168.0, 0.5, 2, 7 + 2000, hidden, per_step) for _ in range(steps)]
    value = sum(v["value"] for v in vals) / len(vals)
    line = {
        "impl": "reference", "metric": "fwd+bwd grads/s (smoothed form)", "value": value, "unit": "grads/s",
        "n_gpus": 1, "steps": steps, "warmup": warmup, "ms_per_step": 1e3 / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generator, procell/calibrate.py problem_inputs)",
        "config": {"workload": "calibration: 256 bins, 1e5 cells, 3 types, t_max 168, h 0.5, 2 lineages per cell",
                   "note": "the reference has no smoothed form; this is its C++ restatement on all host cores"},
        "cpu_baseline": {"value": value, "unit": "grads/s", "cores": vals[-1]["cores"], "kind": "port",
                         "sample": vals[-1]["sample"]},
        "e2e": {"value": value, "unit": "grads/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    return line


def run_calibration(args):
    """Smoothed form alone: fwd+bwd candidate-gradients per second at 256 candidates, and
    gradient-based calibration against particle swarms to equal loss."""
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if rank != 0 and world > 1:
        return 0
    import build as pkg_build
    pkg_build.build()
    from procell import Engine
    eng = Engine(local)
    line = measure_calibration(eng, local, args.steps, args.warmup,
                               None if args.no_cpu_baseline else args.cpu_seconds,
                               pso_seconds=30.0, extra_seeds=(8, 9, 10, 11), extra_pso_seconds=10.0)
    print(json.dumps(line), flush=True)
    return 0


def measure_calibration(eng, local, steps, warmup, cpu_seconds, pso_seconds, extra_seeds, extra_pso_seconds):
    """The calibration workload's line: `steps` timed forward + loss gradient + adjoint
    passes for 256 candidates (and the same end to end from pinned host memory), one
    Jacobian and one Gauss-Newton pass, the race to equal loss on the configured input
    (seed 7, every search, swarm budgets of pso_seconds) and on `extra_seeds`
    (Levenberg-Marquardt against the plain-simulator swarm only), each scored on the
    accurate smoothed loss and on the model-neutral plain-simulator loss."""
    import torch
    from procell import calibrate as cb
    prob = cb.Problem(eng, seed=7)
    C = 256
    theta = prob.start(C, 7)
    stream = torch.cuda.current_stream()

    def step(th):
        P = prob.params(th)
        E = prob.smooth.forward(P)
        r = torch.log1p(E) - prob.target_log  # residuals log(1 + E_v) - log(1 + target_v)
        gE = 2.0 * r / (1.0 + E)
        return prob.smooth.backward(P, gE), (r * r).sum(dim=1)

    for _ in range(warmup):
        step(theta)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        g, L = step(theta)
    e1.record(stream)
    torch.cuda.synchronize()
    eager_ms = e0.elapsed_time(e1)
    # the same step captured once into a CUDA graph and replayed, as the Levenberg-Marquardt
    # harness runs its iterations: the library's six kernels and the loss arithmetic without
    # a host launch each (checked bit for bit against the eager step)
    th_static = theta.clone()
    graph, graph_note = None, None
    try:
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            step(th_static)  # library scratch allocated outside the capture
        torch.cuda.current_stream().wait_stream(side)
        cg = torch.cuda.CUDAGraph()
        with torch.cuda.graph(cg):
            g_static, L_static = step(th_static)
        cg.replay()
        g_ref, L_ref = step(th_static)
        torch.cuda.synchronize()
        if torch.equal(g_static, g_ref) and torch.equal(L_static, L_ref):
            graph = cg
        else:
            graph_note = "graph replay differs from the eager step; eager timings reported"
    except Exception as ex:  # capture unavailable: the eager loop stands
        graph_note = "no graph: " + repr(ex)[:200]
    elapsed_ms = eager_ms
    if graph is not None:
        for _ in range(warmup):
            graph.replay()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            graph.replay()
        e1.record(stream)
        torch.cuda.synchronize()
        elapsed_ms = e0.elapsed_time(e1)
    # end to end: parameters from pinned host memory, gradients and losses back to the host
    host_theta = theta.cpu().pin_memory()
    out_g = torch.empty((C, prob.n_types, 3), dtype=torch.float64).pin_memory()
    out_l = torch.empty(C, dtype=torch.float64).pin_memory()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        if graph is not None:
            th_static.copy_(host_theta, non_blocking=True)
            graph.replay()
            g, L = g_static, L_static
        else:
            th = host_theta.to("cuda", non_blocking=True)
            g, L = step(th)
        out_g.copy_(g, non_blocking=True)
        out_l.copy_(L, non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    clk = clocks.stop()
    h2d = host_theta.numel() * 8
    d2h = (out_g.numel() + out_l.numel()) * 8
    # one pass of the forward-mode Jacobian kernel (expected counts and d/d parameters)
    P0 = prob.params(theta)
    prob.smooth.jacobian(P0)
    j0, j1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    j0.record(stream)
    for _ in range(steps):
        prob.smooth.jacobian(P0)
    j1.record(stream)
    torch.cuda.synchronize()
    jac_ms = j0.elapsed_time(j1) / steps
    # loss and its gradient (plus J^T J) by forward mode: one Gauss-Newton pass
    prob.smooth.gauss_newton(P0, prob.target)
    j0.record(stream)
    for _ in range(steps):
        prob.smooth.gauss_newton(P0, prob.target)
    j1.record(stream)
    torch.cuda.synchronize()
    gn_ms = j0.elapsed_time(j1) / steps
    comp = cb.compare(eng, candidates=C, seed=7, pso_seconds=pso_seconds)
    comp.pop("traces", None)
    others = []
    for sd in extra_seeds:
        c = cb.compare(eng, candidates=C, seed=sd, pso_seconds=extra_pso_seconds, full=False)
        c.pop("traces", None)
        others.append({"seed": sd, "speedup_accurate": c["speedup"], "equal_loss_accurate": c["equal_loss"],
                       "lm_best_accurate": c["lm"]["best_accurate_loss"],
                       "pso_plain_best_accurate": c["pso_plain"]["best_accurate_loss"],
                       "speedup_neutral": c["model_neutral"]["speedup"],
                       "equal_loss_neutral": c["model_neutral"]["equal_loss"],
                       "lm_best_neutral": c["model_neutral"]["lm_best"],
                       "pso_plain_best_neutral": c["model_neutral"]["pso_plain_best"],
                       "neutral_at_hidden": c["model_neutral"]["plain_loss_at_hidden"],
                       "lm_plain_neutral": c["model_neutral"]["lm_plain"],
                       "levels_neutral": c["model_neutral"]["levels"]})
    cpu = None
    if cpu_seconds:
        cpu = cpu_smooth_sample(prob.bins, prob.phi, prob.t_max, prob.smooth_h, prob.smooth_paths,
                                prob.smooth_seed, prob.params(theta[:1]).detach().cpu().numpy(),
                                cpu_seconds)
    value = C * steps / (elapsed_ms * 1e-3)
    hbm, peak_kind = peaks()
    # the smoothed kernels are bound by instruction issue (no FP64 left in the lineage walks,
    # a few MB of inputs and outputs): warp instructions of one forward + adjoint for these
    # 256 candidates (ncu, profiles/) against four issue slots per SM per cycle
    ipp = None
    try:
        with open(os.path.join(ROOT, "profiles", "smooth_instructions_per_pass.txt")) as fh:
            ipp = float(fh.read().split()[0])
    except (OSError, ValueError, IndexError):
        pass
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    issue_peak = 4.0 * sms * clk["sm_mhz"] * 1e6 if clk.get("sm_mhz") else None
    issue_rate = ipp * steps / (elapsed_ms * 1e-3) if ipp else None
    line = {
        "metric": "fwd+bwd grads/s (smoothed form)",
        "value": value,
        "unit": "grads/s",
        "n_gpus": 1,
        "steps": steps,
        "warmup": warmup,
        "ms_per_step": elapsed_ms / steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded generator, procell/calibrate.py Problem)",
        "config": {"workload": "calibration: 256 bins, 1e5 cells, 3 types, %d candidates, t_max 168, h 0.5, "
                               "%d lineages per cell; a step = smoothed forward + loss gradient + adjoint"
                               % (C, prob.smooth_paths),
                   "launch": ("the step replayed from a CUDA graph captured once (bit-identical to the eager "
                              "step)" if graph is not None else "eager: " + str(graph_note)),
                   "l2": "inputs (bins, parameters) are a few MB; the kernels are compute bound"},
        "eager": {"ms_per_step": eager_ms / steps, "grads_per_s": C * steps / (eager_ms * 1e-3),
                  "what": "the same step launched call by call (library calls and torch operations)"},
        "calibration": comp,
        "calibration_other_seeds": {
            "swarm_seconds": extra_pso_seconds, "results": others,
            "what": "problem_inputs(seed) for each seed: Levenberg-Marquardt against the plain-simulator swarm, "
                    "equal-loss ratio on the accurate smoothed loss and on the model-neutral plain loss"},
        "jacobian_pass": {"ms": jac_ms, "candidates_per_s": C / (jac_ms * 1e-3),
                          "what": "expected counts and their Jacobian in (ratio, mean, sd) for %d candidates" % C},
        "forward_mode": {"ms": gn_ms, "grads_per_s": C / (gn_ms * 1e-3),
                         "what": "loss, its gradient (J^T r) and J^T J of %d candidates in one forward-mode "
                                 "pass (pc_smooth_gauss_newton); the value above is forward + adjoint" % C},
        "e2e": {"value": C * steps / e2e_s, "unit": "grads/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "issue", "achieved": issue_rate, "peak": issue_peak,
                     "unit": "warp instructions/s",
                     "frac": (issue_rate / issue_peak) if (issue_rate and issue_peak) else None,
                     "traffic": None, "peak_source": "4 issue slots x %d SMs x sampled SM clock" % sms,
                     "kernel": "k_smooth",
                     "note": "%s warp instructions per forward + adjoint of %d candidates (ncu, "
                             "profiles/smooth_instructions_per_pass.txt); the lineage walks run on the FP32 "
                             "pipe, inputs and outputs are a few MB" % (ipp, C)},
        "gpu_launches": 6 * steps,  # per step: order, forward, merge; order, adjoint, sum
        "clocks": clk,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    return line


def batched_traffic(divisions, launches):
    """Measured DRAM bytes per division of the batched sweeps (ncu, profiles/) x divisions
    per launch."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic_per_division_batched.txt")) as fh:
            return float(fh.read().split()[0]) * divisions / max(1, launches)
    except (OSError, ValueError, IndexError):
        return None


def cpu_batched_sample(instances, seconds):
    """Oracle instances/s on instances drawn at random (seeded) until `seconds` pass."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    cores = os.cpu_count() or 1
    order = np.random.default_rng(0).permutation(len(instances))
    t0 = time.perf_counter()
    done = 0
    for i in order:
        bins, types, t_max, phi, seed = instances[i]
        rows = list(zip(bins[0].tolist(), bins[1].tolist()))
        oracle.simulate(rows, types, t_max, phi, seed=seed, nthreads=cores)
        done += 1
        if time.perf_counter() - t0 > seconds:
            break
    cs = time.perf_counter() - t0
    return {"value": done / cs, "unit": "instances/s", "cores": cores, "kind": "port",
            "sample": "oracle on %d instances drawn at random from the %d (%.1f s), %d threads"
                      % (done, len(instances), cs, cores)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["small", "medium", "large", "batched", "calibration"], default="large")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (default configuration)")
    ap.add_argument("--split", choices=["replicas", "roots"], default="replicas",
                    help="N GPUs: independent replicas (weak scaling, default) or one input split by "
                         "initial-cell ranges with one sum of the counts per step (strong scaling)")
    ap.add_argument("--no-forms", action="store_true",
                    help="plain workload only: skip the batched and calibration forms nested in its line")
    args = ap.parse_args()
    if args.warmup < 3:
        print("warning: --warmup < 3 violates the timing rules", file=sys.stderr)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "calibration":
        return run_calibration(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
