"""Sharded runs over several processes (one GPU each): initial cells split into contiguous
ranges, one plan per rank restricted to its range (pc_plan_set_roots), and a single
element-wise uint64 sum of the per-(value, type) counts. Every initial cell's subtree is
independent (its random stream is keyed by the cell's index and lineage), so the summed
histogram is bit-identical to a one-process run, whatever the number of ranks.

    torchrun --nproc-per-node N script.py      # each rank:
    res = simulate_sharded(engine_shard(Engine(local_rank), bins, types, t_max, phi, seed),
                           total_cells(bins),
                           split=lambda r, n: shard_range_weighted(bins, types, t_max, phi, r, n))
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

STAT_KEYS = ("roots", "divisions", "leaves", "uncounted", "vanished")


def shard_range(total: int, rank: int, world: int):
    """Contiguous, balanced range [lo, hi) of `total` initial cells for `rank`."""
    lo = total * rank // world
    hi = total * (rank + 1) // world
    return lo, hi


def phi_cap(value: float, phi: float, limit: int = 4096) -> int:
    """Generations a cell of this bin may divide: halvings with value / 2 > phi
    (the division test of src/simulation/proliferation.cu:323)."""
    c, f = 0, float(value)
    while f / 2 > phi and c < limit:
        f /= 2
        c += 1
    return c


def cell_work(bins, types, t_max, phi=None):
    """Expected divisions per initial cell of each row of `bins` (rows with frequency 0
    included, weight 0): sum over types of ratio * (2^min(cap, t_max // mean) - 1), the
    full binary tree that the phi cap and the mean division time allow, plus one for the
    root itself. An estimate for balancing shards only; results never depend on it."""
    if phi is None:
        phi = min(float(v) for v, f in bins if int(f) > 0)
    gens = [(float(r), int(t_max // m) if m > 0 else 0) for r, m, _ in types]
    out = []
    for v, f in bins:
        if int(f) == 0:
            out.append(0.0)
            continue
        cap = phi_cap(v, phi)
        out.append(1.0 + sum(r * (2.0 ** min(cap, g, 60) - 1.0) for r, g in gens))
    return out


def shard_range_weighted(bins, types, t_max, phi, rank: int, world: int):
    """Contiguous range [lo, hi) of initial cells (numbered in file order, as pc_plan_set_roots
    counts them) holding about 1/world of the expected work (cell_work) for `rank`. Cuts may
    fall inside a bin; any split gives a bit-identical summed histogram."""
    w = cell_work(bins, types, t_max, phi)
    freqs = [int(f) for _, f in bins]
    total_work = sum(wi * fi for wi, fi in zip(w, freqs))
    total = sum(freqs)
    if total_work <= 0.0:
        return shard_range(total, rank, world)

    def cut(k):  # first cell index at which the cumulative work reaches k/world of the total
        if k <= 0:
            return 0
        if k >= world:
            return total
        target = total_work * k / world
        acc, cell = 0.0, 0
        for wi, fi in zip(w, freqs):
            if fi == 0:
                continue
            if acc + wi * fi >= target:
                return cell + min(fi, int(math.ceil((target - acc) / wi)) if wi > 0 else fi)
            acc += wi * fi
            cell += fi
        return total
    return cut(rank), cut(rank + 1)


def total_cells(bins) -> int:
    return int(sum(int(f) for _, f in bins))


@dataclass
class ShardResult:
    values: np.ndarray            # float64 [V]
    per_type: np.ndarray          # uint64 [V, K]
    stats: dict = field(default_factory=dict)

    @property
    def totals(self):
        return self.per_type.sum(axis=1, dtype=np.uint64)


def engine_shard(engine, bins, types, t_max, phi, seed):
    """compute(lo, hi) on this rank's GPU through the C ABI."""
    def compute(lo, hi):
        p = engine.plan(bins, types, t_max, phi, seed)
        try:
            p.set_roots(lo, hi)
            p.run()
            r = p.result()
        finally:
            p.close()
        return ShardResult(r.values, r.per_type, {k: int(r.stats[k]) for k in STAT_KEYS}
                           | {"max_generation": int(r.stats["max_generation"])})
    return compute


def simulate_sharded(compute, total: int, group=None, split=None) -> ShardResult:
    """Run this rank's shard with compute(lo, hi) -> ShardResult and sum all ranks' counts
    (torch.distributed all_reduce; gloo on CPU tensors, NCCL on CUDA tensors). Every rank
    returns the full histogram. split(rank, world) -> (lo, hi) chooses the ranges (e.g. a
    shard_range_weighted closure); by default equal numbers of initial cells."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    lo, hi = split(rank, world) if split else shard_range(total, rank, world)
    mine = compute(lo, hi)
    if world == 1:
        return mine
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    counts = torch.from_numpy(mine.per_type.astype(np.int64)).to(dev)
    stats = torch.tensor([mine.stats[k] for k in STAT_KEYS], dtype=torch.int64, device=dev)
    gen = torch.tensor([mine.stats.get("max_generation", 0)], dtype=torch.int64, device=dev)
    dist.all_reduce(counts, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(stats, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(gen, op=dist.ReduceOp.MAX, group=group)
    st = {k: int(v) for k, v in zip(STAT_KEYS, stats.cpu().tolist())}
    st["max_generation"] = int(gen.item())
    return ShardResult(mine.values, counts.cpu().numpy().astype(np.uint64), st)
