"""Sharded runs over several processes (one GPU each): initial cells split into contiguous
ranges, one plan per rank restricted to its range (pc_plan_set_roots), and a single
element-wise uint64 sum of the per-(value, type) counts. Every initial cell's subtree is
independent (its random stream is keyed by the cell's index and lineage), so the summed
histogram is bit-identical to a one-process run, whatever the number of ranks.

    torchrun --nproc-per-node N script.py      # each rank:
    res = simulate_sharded(engine_shard(Engine(local_rank), bins, types, t_max, phi, seed),
                           total_cells(bins))
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

STAT_KEYS = ("roots", "divisions", "leaves", "uncounted", "vanished")


def shard_range(total: int, rank: int, world: int):
    """Contiguous, balanced range [lo, hi) of `total` initial cells for `rank`."""
    lo = total * rank // world
    hi = total * (rank + 1) // world
    return lo, hi


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


def simulate_sharded(compute, total: int, group=None) -> ShardResult:
    """Run this rank's shard with compute(lo, hi) -> ShardResult and sum all ranks' counts
    (torch.distributed all_reduce; gloo on CPU tensors, NCCL on CUDA tensors). Every rank
    returns the full histogram."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    lo, hi = shard_range(total, rank, world)
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
