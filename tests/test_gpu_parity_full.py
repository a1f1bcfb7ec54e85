"""Oracle parity at the benchmark's own sizes and over long runs, through the C ABI.

* P-1M (1,048,576 spheres, N = 1024, rigid) for 1,000 frames: keys, permutation,
  cell ranges, positions and packed velocity / force bit-exact against the oracle
  at frames 1, 2, 11, 100, 201, 500 and 1,000 - the late frames run a settled
  floor layer where every sphere has several contacts per frame.  The
  penetration-depth and kinetic-energy statistics (bevy_millions_ball_gb300.stats)
  are compared as well, under the bounds stated there (contact count 5 %, mean
  and 99th-percentile depth 10 %, maximum depth 50 %, kinetic energy 5 %), which
  bit-exact states meet with zero difference.
* P-4M (4,194,304 spheres in 16 Gaussian clusters, N = 2048, spring k = 1000,
  c = 5): bit-exact at frames 1, 2, 3, 12 and 30.
* A batch of 20 mixed scenes compared with the oracle scene by scene (not with
  a lone GPU world), including scenes held for a few frames.

What these restate: physics.wgsl:57-97 (frame) and :119-169 (contacts, jitter).
"""

import numpy as np
import pytest

import oracle
from bevy_millions_ball_gb300 import Batch, World, scenes, stats
from tests.test_gpu_batch import mixed_scenes
from tests.test_gpu_world import INV, TOL_1, TOL_10, compare, run_pair

pytestmark = pytest.mark.gpu


def test_p1m_long_run_bit_exact_with_statistics(built_lib, cuda):
    pytest.importorskip("scipy")
    sc = scenes.workload("P-1M")
    dt = scenes.quantized_dt(sc.plugin.time_delta)
    seen = {}
    with World(sc.plugin) as w:
        ow = oracle.OracleWorld(sc.plugin.to_c())
        w.set_state(sc.pos_scale, sc.vfme)
        ow.set_state(sc.pos_scale, sc.vfme)
        done = 0
        for cp in [1, 2, 11, 100, 201, 500, 1000]:
            w.step(cp - done)
            ow.step(cp - done)
            done = cp
            w.sync()
            compare(w, ow, cp, TOL_1 if cp == 2 else (TOL_10 if cp == 11 else None))
            if cp >= 201:
                p, q = w.get_state()
                rp, rq = ow.get_state()
                a, b = stats.contact_stats(p, q, dt), stats.contact_stats(rp, rq, dt)
                cmp = stats.compare(a, b)
                assert all(ok for _, _, ok in cmp.values()), (cp, cmp)
                seen[cp] = a
        ow.close()
    # the late frames are the contact-heavy regime the bench runs into
    assert seen[1000]["contacts"] > 100_000 and seen[1000]["kinetic_energy"] > 0.0


def test_p4m_clustered_spring_bit_exact(built_lib, cuda):
    """The 4,194,304-sphere clustered spring workload at full size: cells near the
    cluster centres hold ~100 spheres (crowded-warp walk, bands too wide to stage,
    large fixup cells)."""
    run_pair(scenes.workload("P-4M"), 30, [1, 2, 3, 12, 30])


def _compare_scene(b: Batch, i: int, ow: "oracle.OracleWorld", what: str):
    p, q = b.get_state(i)
    rp, rq = ow.get_state()
    d, rd = b.debug(i), ow.debug()
    np.testing.assert_array_equal(d["keys"], rd["keys"], err_msg=f"{what}: keys")
    np.testing.assert_array_equal(d["perm"], rd["perm"], err_msg=f"{what}: perm")
    np.testing.assert_array_equal(d["start"], rd["start"], err_msg=f"{what}: start")
    full = rd["start"] != INV
    np.testing.assert_array_equal(d["close"][full], rd["close"][full], err_msg=f"{what}: close")
    np.testing.assert_array_equal(p.view(np.uint32), rp.view(np.uint32), err_msg=f"{what}: positions")
    np.testing.assert_array_equal(q, rq, err_msg=f"{what}: vfme")


def test_batch_scenes_match_the_oracle(built_lib, cuda):
    """Each scene of a 20-scene batch (sizes 200-30,000, rigid and spring, mixed
    heights and restitution) against its own oracle world: the batched kernels
    (per-scene parameters read in place, scene-local jitter index, per-scene
    buffer parity, held scenes) checked directly, not through a lone GPU world."""
    scs = mixed_scenes(20, seed=5, n_min=200, n_max=30_000)
    ows = [oracle.OracleWorld(s.plugin.to_c()) for s in scs]
    held = {3, 7, 12}
    with Batch([s.plugin for s in scs]) as b:
        for i, s in enumerate(scs):
            b.set_state(i, s.pos_scale, s.vfme)
            ows[i].set_state(s.pos_scale, s.vfme)

        def step(k, skip=()):
            b.step(k)
            for i, ow in enumerate(ows):
                if i not in skip:
                    ow.step(k)

        step(1)  # INIT
        for i, ow in enumerate(ows):
            _compare_scene(b, i, ow, f"scene {i}, frame 1")
        step(10)
        for i in held:
            b.set_active(i, False)
        step(5, skip=held)  # held scenes keep state, keys and order
        for i in held:
            b.set_active(i, True)
        step(19)
        b.sync()
        for i, ow in enumerate(ows):
            _compare_scene(b, i, ow, f"scene {i}, frame {ow.time}")
            assert b.time(i) == ow.time
    for ow in ows:
        ow.close()
