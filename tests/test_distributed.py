"""Sharded multi-process runs: world_size-2 gloo ranks on CPU.

Each rank computes its contiguous range of initial cells (here with the oracle, the CPU
restatement, standing in for the rank's GPU) and procell.distributed sums the counts with
one all_reduce. The sum must equal a one-process run bit for bit, for any world size.
"""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _oracle_compute(bins, types, t_max, phi, seed):
    import oracle
    from procell.distributed import STAT_KEYS, ShardResult

    def compute(lo, hi):
        r = oracle.simulate(bins, types, t_max, phi, seed=seed, root_begin=lo, root_end=hi, nthreads=2)
        st = {k: r.stats[k] for k in STAT_KEYS}
        st["max_generation"] = r.stats["max_gen"]
        return ShardResult(r.values, r.per_type, st)
    return compute


def _rank_main(rank, world, port, case, out_dir, weighted=False):
    sys.path[:0] = [os.path.join(ROOT, "cuda-pro-cell_gb300"), os.path.join(ROOT, "oracle")]
    import torch.distributed as dist
    from procell.distributed import shard_range_weighted, simulate_sharded, total_cells
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bins, types, t_max, phi, seed = case
        split = (lambda r, n: shard_range_weighted(bins, types, t_max, phi, r, n)) if weighted else None
        res = simulate_sharded(_oracle_compute(bins, types, t_max, phi, seed), total_cells(bins), split=split)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), values=res.values, per_type=res.per_type,
                 stats=np.array([res.stats[k] for k in ("roots", "divisions", "leaves", "uncounted", "vanished",
                                                        "max_generation")], np.int64))
    finally:
        dist.destroy_process_group()


CASE = ([(float(v), int(f)) for v, f in zip(np.geomspace(2.0, 5000.0, 24), [30, 0, 12, 50] * 6)],
        [(0.5, 30.0, 9.0), (0.3, 45.0, 12.0), (0.2, -1.0, -1.0)], 120.0, None, 77)


@pytest.mark.parametrize("world,weighted", [(2, False), (3, False), (2, True), (3, True)])
def test_gloo_shards_sum_to_full_run(oracle_lib, tmp_path, world, weighted):
    bins, types, t_max, phi, seed = CASE
    full = oracle_lib.simulate(bins, types, t_max, phi, seed=seed, nthreads=2)
    mp.start_processes(_rank_main, args=(world, _free_port(), CASE, str(tmp_path), weighted), nprocs=world,
                       join=True, start_method="spawn")
    for r in range(world):
        d = np.load(tmp_path / f"rank{r}.npz")
        assert np.array_equal(d["values"], full.values)
        assert np.array_equal(d["per_type"], full.per_type)
        st = d["stats"]
        assert list(st[:5]) == [full.stats[k] for k in ("roots", "divisions", "leaves", "uncounted", "vanished")]
        assert st[5] == full.stats["max_gen"]


def test_shard_ranges_cover_exactly():
    from procell.distributed import shard_range
    for total in (0, 1, 7, 1000, 10 ** 7 + 3):
        for world in (1, 2, 3, 8):
            ranges = [shard_range(total, r, world) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == total
            assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
            assert max(h - l for l, h in ranges) - min(h - l for l, h in ranges) <= 1


def test_weighted_shard_ranges_cover_exactly():
    import procell.configs as cfg
    from procell.distributed import shard_range_weighted, total_cells
    for w in (cfg.small(), cfg.medium()):
        for world in (1, 2, 3, 8):
            r = [shard_range_weighted(w.bins, w.types, w.t_max, w.phi, k, world) for k in range(world)]
            assert r[0][0] == 0 and r[-1][1] == total_cells(w.bins)
            assert all(a[1] == b[0] and a[0] <= a[1] for a, b in zip(r, r[1:]))


def test_weighted_split_balances_skewed_work(oracle_lib):
    """Bins sorted by value put cells with shallow trees first and deep ones last; equal
    numbers of initial cells then give very unequal shards, the work-weighted split does
    not (divisions per shard counted by the oracle)."""
    from procell.distributed import shard_range, shard_range_weighted, total_cells
    bins = [(float(v), 300) for v in np.geomspace(2.0, 2.0 ** 12, 48)]
    types = [(0.6, 20.0, 5.0), (0.4, 30.0, 6.0)]
    t_max, phi, world = 160.0, 1.0, 4

    def spread(ranges):
        d = [oracle_lib.simulate(bins, types, t_max, phi, seed=3, root_begin=lo, root_end=hi,
                                 nthreads=2).stats["divisions"] for lo, hi in ranges]
        return max(d) / max(1, min(d))

    n = total_cells(bins)
    equal = spread([shard_range(n, k, world) for k in range(world)])
    weighted = spread([shard_range_weighted(bins, types, t_max, phi, k, world) for k in range(world)])
    assert weighted < 1.5 < equal, (weighted, equal)


@pytest.mark.gpu
def test_engine_shards_sum_to_full_run(engine):
    import procell.configs as cfg
    from procell.distributed import engine_shard, shard_range, total_cells
    w = cfg.small()
    compute = engine_shard(engine, w.bins, w.types, w.t_max, w.phi, w.seed)
    total = total_cells(w.bins)
    parts = [compute(*shard_range(total, r, 3)) for r in range(3)]
    full = engine.simulate(w.bins, w.types, w.t_max, w.phi, w.seed)
    assert np.array_equal(sum(p.per_type for p in parts), full.per_type)
    assert sum(p.stats["divisions"] for p in parts) == full.stats["divisions"]


@pytest.mark.gpu
def test_simulate_shard_and_accumulate_through_the_c_abi(engine):
    """pc_simulate_shard over four uneven shards, added with pc_histogram_accumulate, equals
    pc_simulate on the whole input bit for bit (the small workload)."""
    import ctypes
    import procell.configs as cfg
    from procell import _lib
    w = cfg.small()
    b, t = _lib.bins_numpy(w.bins), _lib.types_numpy(w.types)
    bp, tp = b.ctypes.data_as(ctypes.POINTER(_lib.Bin)), t.ctypes.data_as(ctypes.POINTER(_lib.CellType))
    L = engine.L
    full = _lib.Histogram()
    engine._check(L.pc_simulate(engine.ctx, bp, len(b), tp, len(t), w.t_max, w.phi, w.seed, ctypes.byref(full)))
    n = int(b["frequency"].sum())
    cuts = [0, 1, n // 5, n // 2 + 7, n]
    acc = None
    for lo, hi in zip(cuts, cuts[1:]):
        h = _lib.Histogram()
        engine._check(L.pc_simulate_shard(engine.ctx, bp, len(b), tp, len(t), w.t_max, w.phi, w.seed, lo, hi,
                                          ctypes.byref(h)))
        if acc is None:
            acc = h
        else:
            assert L.pc_histogram_accumulate(ctypes.byref(acc), ctypes.byref(h)) == 0
            L.pc_histogram_free(ctypes.byref(h))
    fv, ft, fp, fs = _lib.histogram_to_numpy(full)
    av, at, ap, ast = _lib.histogram_to_numpy(acc)
    L.pc_histogram_free(ctypes.byref(full))
    L.pc_histogram_free(ctypes.byref(acc))
    assert np.array_equal(fv, av) and np.array_equal(ft, at) and np.array_equal(fp, ap)
    for k in ("roots", "divisions", "leaves", "uncounted", "vanished", "max_generation"):
        assert fs[k] == ast[k], k
