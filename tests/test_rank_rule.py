"""The rank-placement rule, checked on the CPU against a stable sort.

The reference orders each frame's spheres by a stable radix sort of their cell
keys (bevy_radix_sort, called at src/physics/mod.rs:880-890).  Rank placement
(MB_SORT_RANK, the GPU's default) places a sphere at its new cell's offset plus
the number of spheres of that cell that precede it in its old 3 x 3 cell
neighbourhood, plus the far moves (spheres that moved more than one cell) of
that cell that precede it.  This test restates that rule in numpy and shows it
equals the stable sort on generated frames: an old order sorted by cell, moves
of at most one cell, far moves, grid edges and crowded cells.  It needs no GPU.
"""

import numpy as np
import pytest


def stable_order(keys):
    return np.argsort(keys, kind="stable")


def rank_placement(new_keys, old_offs, N):
    """Slot of each input sphere by the rule (input = the old sorted order)."""
    n = new_keys.size
    C = N * N
    counts = np.bincount(new_keys, minlength=C)
    offs = np.concatenate([[0], np.cumsum(counts)])
    old_cell = np.searchsorted(old_offs, np.arange(n), side="right") - 1
    ox, oz = old_cell % N, old_cell // N
    nx, nz = new_keys % N, new_keys // N
    far = (np.abs(nx - ox) > 1) | (np.abs(nz - oz) > 1)
    far_slots = np.nonzero(far)[0]
    slot = np.empty(n, np.int64)
    for i in range(n):
        k = int(new_keys[i])
        kx, kz = k % N, k // N
        c0, c1 = max(kx - 1, 0), min(kx + 1, N - 1) + 1
        cnt = 0
        for r in range(max(kz - 1, 0), min(kz + 1, N - 1) + 1):
            lo, hi = old_offs[r * N + c0], min(old_offs[r * N + c1], i)
            if hi > lo:
                cnt += int(np.count_nonzero(new_keys[lo:hi] == k))
        cnt += int(np.count_nonzero((new_keys[far_slots] == k) & (far_slots < i)))
        slot[i] = offs[k] + cnt
    return slot, int(far.sum())


def frame(rng, n, N, far_moves, crowd=False):
    """An old order (sorted by cell) and each sphere's new cell."""
    C = N * N
    if crowd:
        old_keys = np.sort(rng.integers(0, max(C // 16, 1), n) * 3 % C)
    else:
        old_keys = np.sort(rng.integers(0, C, n))
    old_offs = np.concatenate([[0], np.cumsum(np.bincount(old_keys, minlength=C))])
    x, z = old_keys % N, old_keys // N
    x = np.clip(x + rng.integers(-1, 2, n) * (rng.random(n) < 0.3), 0, N - 1)
    z = np.clip(z + rng.integers(-1, 2, n) * (rng.random(n) < 0.3), 0, N - 1)
    jump = rng.choice(n, far_moves, replace=False) if far_moves else np.array([], np.int64)
    x[jump] = rng.integers(0, N, jump.size)
    z[jump] = rng.integers(0, N, jump.size)
    return (z * N + x).astype(np.int64), old_offs


@pytest.mark.parametrize("case", ["sparse", "dense", "crowded", "edges", "far"])
def test_rank_rule_equals_stable_sort(case):
    rng = np.random.default_rng(["sparse", "dense", "crowded", "edges", "far"].index(case) + 7)
    n, N, far_moves, crowd = {"sparse": (600, 48, 0, False), "dense": (3000, 40, 0, False),
                              "crowded": (2500, 32, 0, True), "edges": (800, 4, 0, False),
                              "far": (2000, 40, 60, False)}[case]
    new_keys, old_offs = frame(rng, n, N, far_moves, crowd)
    slot, far = rank_placement(new_keys, old_offs, N)
    order = np.empty(n, np.int64)
    order[slot] = np.arange(n)
    np.testing.assert_array_equal(order, stable_order(new_keys))
    if case == "far":
        assert far > 0
