"""Rank placement (MB_SORT_RANK) against the oracle, bit-exact.

After the first sort, a frame's input is the previous frame's sorted order, and
each sphere's slot is its new cell's offset plus the number of spheres of that
cell before it in its old 3 x 3 cell neighbourhood; spheres that moved more than
one cell (far moves) are listed by the physics pass and ranked from the list
(up to 256 per frame), beyond which the frame claims slots and fixes cells like
MB_SORT_COUNTING.  The reference has one order for all of this: the stable radix
sort of the keys (bevy_radix_sort, called at src/physics/mod.rs:880-890), whose
start/close tables spatial_hashing.wgsl:29-70 builds; the oracle restates both.
"""

import numpy as np
import pytest

import oracle
from bevy_millions_ball_gb300 import Batch, MbError, World, _abi, pack_vfme, scenes, unpack_vfme
from tests.test_gpu_batch import mixed_scenes
from tests.test_gpu_parity_full import _compare_scene
from tests.test_gpu_world import compare, run_pair

pytestmark = pytest.mark.gpu
RANK = {"sort_algorithm": _abi.MB_SORT_RANK}


def fast_scene(m: int, speed: float, seed: int = 5, n: int = 65_536, grids: int = 256):
    """A uniform scene in which m spheres move `speed` cells per frame along x/z."""
    sc = scenes.plain_uniform(n, grids, seed=seed)
    rng = np.random.default_rng(seed + 1)
    v, f, mass = unpack_vfme(sc.vfme)
    idx = rng.choice(sc.n, m, replace=False)
    ang = rng.uniform(0.0, 2.0 * np.pi, m)
    v[idx, 0] = speed * np.cos(ang)
    v[idx, 2] = speed * np.sin(ang)
    sc.vfme = pack_vfme(v, f, mass)
    return sc


def _cells(ow: "oracle.OracleWorld", plugin, p):
    c = oracle.quantize(plugin.to_c())
    N, G, H = plugin.number_of_grids_one_dimension, plugin.grid_size, np.float32(c.half_map_size)
    x = np.clip((p[:, 0] + H).astype(np.float64), 0, None).astype(np.uint64) // G
    z = np.clip((p[:, 2] + H).astype(np.float64), 0, None).astype(np.uint64) // G
    return np.minimum(x, N - 1).astype(np.int64), np.minimum(z, N - 1).astype(np.int64)


def run_frame_by_frame(sc, frames, tuning=None):
    """Steps the world and the oracle one frame at a time and compares every
    frame; returns the number of far moves each frame's sort had to place."""
    far = []
    with World(sc.plugin) as w:
        w.set_tuning(**(tuning or RANK))
        ow = oracle.OracleWorld(sc.plugin.to_c())
        w.set_state(sc.pos_scale, sc.vfme)
        ow.set_state(sc.pos_scale, sc.vfme)
        prev = None
        for f in range(1, frames + 1):
            w.step(1)
            ow.step(1)
            compare(w, ow, f)
            p, _ = ow.get_state()
            cx, cz = _cells(ow, sc.plugin, p)
            if prev is not None and f >= 3:
                perm = ow.debug()["perm"]
                ox, oz = prev[0][perm], prev[1][perm]
                far.append(int(((np.abs(cx - ox) > 1) | (np.abs(cz - oz) > 1)).sum()))
            prev = (cx, cz)
    return far


@pytest.mark.parametrize("case", ["small", "clustered", "crowded", "degenerate", "mixed", "sparse", "odd"])
def test_rank_matches_oracle(built_lib, cuda, case):
    """Workload shapes of the claim-and-fixup tests, ranked instead (the
    clustered, crowded and degenerate scenes overflow the far list in some
    frames and so cover the switch between the two paths)."""
    if case == "small":
        run_pair(scenes.workload("P-small"), 101, [1, 2, 3, 11, 50, 101], tuning=RANK)
    elif case == "clustered":
        run_pair(scenes.plain_clustered(262_144, 512, clusters=4, sigma_xz=16.0, seed=9), 40, [1, 2, 3, 11, 40],
                 tuning=RANK)
    elif case == "crowded":
        run_pair(scenes.plain_uniform(51_200, 16, grid_size=1, half_map_height=8, seed=31), 6, [1, 2, 3, 6],
                 tuning=RANK)
    elif case == "degenerate":
        run_pair(scenes.plain_uniform(36_000, 2, grid_size=4, half_map_height=8, seed=32), 4, [1, 2, 3, 4],
                 tuning=RANK)
    elif case == "mixed":
        sc = scenes.plain_uniform(40_000, 128, half_map_height=4, seed=31, spring=True)
        rng = np.random.default_rng(33)
        v, f, _ = unpack_vfme(sc.vfme)
        sc.vfme = pack_vfme(v, f, rng.choice(np.array([0.5, 1.0, 1.5, 2.0, 0.7], np.float32), sc.n))
        sc.pos_scale[:, 3] = rng.choice(np.array([0.3, 0.45, 0.5, 0.6], np.float32), sc.n)
        run_pair(sc, 30, [1, 2, 3, 11, 30], tuning=RANK)
    elif case == "sparse":
        run_pair(scenes.plain_uniform(5_000, 512, seed=13), 25, [1, 2, 3, 11, 25], tuning=RANK)
    else:
        run_pair(scenes.plain_uniform(20_000, 64, grid_size=7, half_map_height=4, seed=47), 14, [1, 2, 3, 14],
                 tuning=RANK)


def test_rank_far_moves_listed(built_lib, cuda):
    """About 40 spheres per frame move more than one cell: every one is ranked
    from the far list (and the cells it lands in counted from it), frame by frame."""
    far = run_frame_by_frame(fast_scene(100, 1.6), 24)
    assert all(0 < k <= 256 for k in far), far


def test_rank_far_list_overflows_midrun(built_lib, cuda):
    """Far moves grow from ~150 to ~270 per frame: frames switch from ranking
    with the list to the claim-and-fixup path once it overflows."""
    far = run_frame_by_frame(fast_scene(150, 2.5), 32)
    assert any(0 < k <= 256 for k in far) and any(k > 256 for k in far), far


@pytest.mark.parametrize("tuning", [{"state_gather": 1}, {"collide_block": 64}, {"collide_block": 256},
                                    {"frames_per_launch": 1}, {"frames_per_launch": 16}, {"scatter_agents": 2},
                                    {"scatter_agents": 4}])
def test_rank_with_other_knobs(built_lib, cuda, tuning):
    """The gather through the permutation, the other physics tiles and chain
    lengths, two and four spheres placed per thread."""
    run_pair(fast_scene(100, 1.6, seed=8), 40, [1, 2, 3, 11, 40], tuning={**RANK, **tuning})


def test_rank_switches_and_settings(built_lib, cuda):
    """Switches between the three sorts, a grid change and a re-upload mid-run."""
    sc = scenes.plain_clustered(120_000, 256, clusters=3, sigma_xz=12.0, seed=19)
    with World(sc.plugin) as w:
        ow = oracle.OracleWorld(sc.plugin.to_c())
        w.set_state(sc.pos_scale, sc.vfme)
        ow.set_state(sc.pos_scale, sc.vfme)
        for alg, k in [(2, 5), (0, 3), (2, 4), (1, 3), (2, 6), (0, 2)]:
            w.set_tuning(sort_algorithm=alg)
            if ow.time:
                compare(w, ow, ow.time)  # the cell ranges follow the sort into its offsets buffer
            w.step(k)
            ow.step(k)
            compare(w, ow, ow.time)
        new = sc.plugin.replace(number_of_grids_one_dimension=128, grid_size=2)
        w.set_settings(new)
        ow.set_settings(new.to_c())
        for k in (1, 1, 5):
            w.step(k)
            ow.step(k)
            compare(w, ow, ow.time)
        w.set_state(sc.pos_scale, sc.vfme)
        ow.set_state(sc.pos_scale, sc.vfme)
        w.step(7)
        ow.step(7)
        compare(w, ow, 7)
        with pytest.raises(MbError):
            w.set_tuning(sort_algorithm=2, frame_kernel=_abi.MB_FRAME_FUSED)  # fused frames claim and fix


def test_rank_full_size_late_frames(built_lib, cuda):
    """The 1,048,576-sphere workload ranked for 300 frames (settled floor, several
    contacts per sphere), compared at frames 3, 100 and 300."""
    run_pair(scenes.workload("P-1M"), 300, [3, 100, 300], tuning=RANK)


@pytest.mark.parametrize("sort", [_abi.MB_SORT_RANK, _abi.MB_SORT_COUNTING])
def test_batch_rank_against_the_oracle(built_lib, cuda, sort):
    """A pool of mixed scenes plus two with fast spheres (far moves listed pool-wide,
    and more than the list holds in some frames): frames in which every scene is
    in LOOP are ranked, frames with a held scene claim and fix, and the switch
    back to ranking starts from a claimed frame; each scene against its own
    oracle world, at several points of the run."""
    scs = mixed_scenes(6, seed=41, n_min=500, n_max=20_000) + [fast_scene(90, 1.6, seed=42, n=16_384, grids=128),
                                                             fast_scene(140, 2.5, seed=43)]
    ows = [oracle.OracleWorld(s.plugin.to_c()) for s in scs]
    with Batch([s.plugin for s in scs]) as b:
        b.set_tuning(sort_algorithm=sort)
        with pytest.raises(MbError):
            b.set_tuning(sort_algorithm=_abi.MB_SORT_ONESWEEP)
        for i, s in enumerate(scs):
            b.set_state(i, s.pos_scale, s.vfme)
            ows[i].set_state(s.pos_scale, s.vfme)

        def step(k, skip=()):
            b.step(k)
            for i, ow in enumerate(ows):
                if i not in skip:
                    ow.step(k)

        def check(what):
            b.sync()
            for i, ow in enumerate(ows):
                _compare_scene(b, i, ow, f"scene {i}, {what}")
                assert b.time(i) == ow.time

        step(1)  # INIT
        step(2)
        check("frame 3")
        step(9)  # a chain of 8 and a single frame
        check("frame 12")
        b.set_active(2, False)
        step(3, skip={2})
        b.set_active(2, True)
        step(1)
        check("after a hold")
        step(17)
        check("late")
    for ow in ows:
        ow.close()
