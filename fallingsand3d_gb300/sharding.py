"""How the batched workload splits over GPUs (one process per GPU).

Worlds are independent, so ranks never exchange simulation data: with weak
scaling every rank steps its own batch (master seed + rank); with strong
scaling a fixed world list is split by greedy longest-processing-time
assignment on cell counts.  Only per-world results (hashes) are gathered.
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

World = Tuple[Tuple[int, int, int], int]  # ((X, Y, Z), seed)


def weak_master(master: int, rank: int) -> int:
    """Master seed of the batch a rank steps under weak scaling."""
    return master + rank


def strong_split(worlds: Sequence[World], world_size: int) -> List[List[int]]:
    """Indices of `worlds` per rank, balancing total cells (LPT greedy);
    ties go to the lowest rank so every process computes the same split."""
    order = sorted(range(len(worlds)), key=lambda i: (-_cells(worlds[i]), i))
    load = [0] * world_size
    parts: List[List[int]] = [[] for _ in range(world_size)]
    for i in order:
        r = min(range(world_size), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += _cells(worlds[i])
    return [sorted(p) for p in parts]


def _cells(w: World) -> int:
    (X, Y, Z), _ = w
    return X * Y * Z
