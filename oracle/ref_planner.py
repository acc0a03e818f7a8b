"""Test infrastructure only: a CPU restatement of the reference binary's host-side planner.

The reference sizes its work from free device memory and launches one CUDA Dynamic
Parallelism tree per iteration. This module restates that arithmetic, without running
anything, to decide which inputs the reference binary can run safely on a GPU:

* utils::max_recursion_depth (src/utils/util.cu:37-74): the deepest doubling whose level
  buffers fit in free memory, times 0.9, at most 24;
* simulation::proliferate (src/simulation/proliferation.cu:26-215): per iteration, the depth
  (with the population split of :101-152 when no depth fits), min(depth, -d);
* run_iteration (:217-284): level i holds `current_size * 2^i` cells of 40 bytes, its size
  computed as uint32_t (:233); the grid is `uint16_t n_blocks = round(0.5 + size / 1024)`
  (:245); cells born at the last level make `still_alive` true and start another iteration
  whose population is that whole level, written or not (:283, :315-349).

An input is safe when the whole run is one iteration (no cell is born at generation
`depth`), every level size is below 2^32, the grid size below 65536 and every level fits in
free memory. Otherwise the reference reads uninitialised level slots as cells (a second
iteration), skips cells (a wrapped grid size) or writes past an allocation that a wrapped
level size made too small; such runs are not attempted.
"""
from __future__ import annotations

import math

CELL_BYTES = 40           # sizeof(simulation::cell), src/simulation/data_types.h:12-19
FLUORESCENCE_BYTES = 16   # sizeof(simulation::fluorescence), data_types.h:29-33
RESULT_BYTES = 24         # sizeof(fluorescence_with_ratio), data_types.h:35-40
MAX_DEPTH = 24            # src/utils/util.cu:6
MAX_TREE_DEPTH = 23       # the -d default, src/io/cmdargs.cpp:6,19
THREADS_PER_BLOCK = 1024  # cudaDeviceProp::maxThreadsPerBlock
MAX_GRID_X = 2 ** 31 - 1  # cudaDeviceProp::maxGridSize[0]


def log_two(n: int) -> int:
    """util.cu:25-28: log(n) / log(2) truncated to uint64."""
    return int(math.log(n) / math.log(2))


def max_recursion_depth(results_size: int, initial_stage_size: int, free_bytes: int) -> int:
    """util.cu:37-74 with the given free memory."""
    mem = initial_stage_size * CELL_BYTES
    final = initial_stage_size
    internal_mem = (final * 2 - 2 * initial_stage_size) * CELL_BYTES
    results_mem = results_size * FLUORESCENCE_BYTES
    if mem * 2 + internal_mem + results_mem > free_bytes:
        return 0
    while mem + internal_mem + results_mem < free_bytes:
        if mem * 2 + internal_mem + results_mem < free_bytes:
            final *= 2
            internal_mem = (final - 2 * initial_stage_size) * CELL_BYTES
        mem *= 2
    depth = log_two(final) - log_two(initial_stage_size)
    depth = int(depth * 0.9)
    return min(depth, MAX_DEPTH)


def n_blocks(size: int) -> int:
    """proliferation.cu:245 before the uint16_t conversion: round(0.5 + size / 1024) with
    integer division (round half away from zero)."""
    return size // THREADS_PER_BLOCK + 1


def first_iteration(n_roots: int, n_values: int, free_bytes: int, n_types: int = 1,
                    track_ratio: bool = False, tree_depth: int = MAX_TREE_DEPTH) -> dict:
    """The first iteration's plan for `n_roots` initial cells and an output value set of
    `n_values` entries, with `free_bytes` free before the run (the results table, the ratio
    arrays and the initial cells are allocated first, proliferation.cu:46-98)."""
    held = n_values * RESULT_BYTES + (n_values * n_types * 4 if track_ratio else 0) + n_roots * CELL_BYTES
    free = free_bytes - held
    size = n_roots
    depth = max_recursion_depth(n_values, size, free)
    split = False
    mult = 2
    proposed = size // mult
    while depth == 0 and proposed > 0:
        # the population split of proliferation.cu:101-152
        depth = max_recursion_depth(n_values, proposed, free)
        if depth > 0:
            cur, blocks = proposed, 0
            for _ in range(depth):
                blocks += n_blocks(cur)
                cur *= 2
            if blocks >= MAX_GRID_X:
                depth = 0
        if depth > 0:
            split = True
            size = proposed
        mult += 1
        proposed = size // mult
    depth = min(depth, tree_depth)
    levels = [size * 2 ** i for i in range(1, depth + 1)]
    return {
        "roots_in_first_population": size,
        "split": split,
        "depth": depth,
        "n_blocks": n_blocks(size),
        "largest_level": levels[-1] if levels else size,
        "level_bytes": sum(levels) * CELL_BYTES,
        "free_bytes": free,
    }


def assess(n_roots: int, n_values: int, max_generation: int, free_bytes: int, n_types: int = 1,
           track_ratio: bool = False) -> dict:
    """Whether the reference binary runs an input safely: the first iteration's plan plus
    the reasons it is unsafe (empty when safe). `max_generation` is the deepest generation
    any cell reaches (the oracle's max_gen for the same input)."""
    it = first_iteration(n_roots, n_values, free_bytes, n_types, track_ratio)
    reasons = []
    if it["depth"] == 0:
        reasons.append("no recursion depth fits in free memory")
    if it["split"]:
        reasons.append("the initial population is split across iterations")
    if max_generation >= it["depth"]:
        reasons.append("cells are born at generation %d = the depth: a second iteration reads the whole "
                       "last level, uninitialised slots included, as cells" % it["depth"])
    if it["n_blocks"] >= 2 ** 16:
        reasons.append("the uint16_t grid size wraps (%d blocks)" % it["n_blocks"])
    if it["largest_level"] >= 2 ** 32:
        reasons.append("a uint32_t level size overflows (%d cells)" % it["largest_level"])
    if it["level_bytes"] > it["free_bytes"]:
        reasons.append("the level buffers exceed free memory")
    it["max_generation"] = max_generation
    it["reasons"] = reasons
    it["safe"] = not reasons
    return it
