"""Scene sharding across GPUs for batching and serving.

Scenes are independent, so N ranks (one process per GPU) each step their own
share in their own batch and nothing is exchanged on the data path: the only
cross-rank traffic is the host-side bookkeeping (who owns which scene), and the
benchmark's barrier / max-over-ranks timing.  Shares are balanced by sphere
count with the longest-processing-time greedy rule (largest scene first, to the
rank with the least spheres so far; ties to the lower rank), which every rank
computes identically from the same size list - no collective needed to agree.
"""

from __future__ import annotations


def partition_by_size(sizes, ranks: int) -> list[list[int]]:
    """Indices of `sizes` per rank (each list ascending); LPT greedy balance."""
    if ranks <= 0:
        raise ValueError("ranks must be positive")
    order = sorted(range(len(sizes)), key=lambda i: (-int(sizes[i]), i))
    load = [0] * ranks
    share: list[list[int]] = [[] for _ in range(ranks)]
    for i in order:
        r = min(range(ranks), key=lambda k: (load[k], k))
        share[r].append(i)
        load[r] += int(sizes[i])
    return [sorted(s) for s in share]


def my_scenes(sizes, rank: int, ranks: int) -> list[int]:
    """This rank's scene indices."""
    return partition_by_size(sizes, ranks)[rank]
