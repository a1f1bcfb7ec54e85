"""Batching and serving: many scenes stepped together must each give exactly the
result of stepping that scene alone (state, keys, permutation, cell ranges)."""

import math

import numpy as np
import pytest

from bevy_millions_ball_gb300 import Batch, MbError, Server, World, _abi, scenes

pytestmark = pytest.mark.gpu
INV = 0xFFFFFFFF


def mixed_scenes(count, seed, n_min=50, n_max=20_000):
    rng = np.random.default_rng(seed)
    out = []
    for s in range(count):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        grids = scenes.next_pow2(math.isqrt(max(n - 1, 0)) + 1)
        spring = bool(s % 2)
        sc = scenes.plain_uniform(n, grids, half_map_height=int(rng.choice([4, 8, 16])),
                                  seed=int(rng.integers(0, 2**31)), spring=spring,
                                  e=float(rng.uniform(0.5, 0.95)), k=400.0, c=2.0)
        sc.plugin = sc.plugin.replace(e_envir=float(rng.uniform(0.5, 0.95)))
        out.append(sc)
    return out


def alone(sc, frames):
    with World(sc.plugin) as w:
        w.set_state(sc.pos_scale, sc.vfme)
        w.step(frames)
        p, q = w.get_state()
        return p, q, w.debug()


def assert_same(batch, idx, ref, what, ref_order=None):
    """State and keys against `ref`; order / cell ranges against `ref_order` (default `ref`)."""
    p, q = batch.get_state(idx)
    rp, rq, rd = ref
    od = (ref_order or ref)[2]
    np.testing.assert_array_equal(p.view(np.uint32), rp.view(np.uint32), err_msg=f"{what}: positions")
    np.testing.assert_array_equal(q, rq, err_msg=f"{what}: vfme")
    d = batch.debug(idx)
    np.testing.assert_array_equal(d["keys"], rd["keys"], err_msg=f"{what}: keys")
    np.testing.assert_array_equal(d["perm"], od["perm"], err_msg=f"{what}: perm")
    np.testing.assert_array_equal(d["start"], od["start"], err_msg=f"{what}: start")
    full = od["start"] != INV
    np.testing.assert_array_equal(d["close"][full], od["close"][full], err_msg=f"{what}: close")


def test_batch_matches_each_scene_alone(built_lib, cuda):
    scs = mixed_scenes(9, seed=1)
    with Batch([s.plugin for s in scs]) as b:
        for i, s in enumerate(scs):
            b.set_state(i, s.pos_scale, s.vfme)
        b.step(1)
        for i, s in enumerate(scs):  # INIT frame: identity order, everyone in cell 0
            assert_same(b, i, alone(s, 1), f"scene {i} after INIT")
        b.step(11)
        b.sync()
        for i, s in enumerate(scs):
            assert b.time(i) == 12
            assert_same(b, i, alone(s, 12), f"scene {i}")


def test_batch_hold_and_late_upload(built_lib, cuda):
    scs = mixed_scenes(5, seed=2)
    extra = mixed_scenes(1, seed=3)[0]
    cap_a = sum(s.n for s in scs) + extra.n
    cap_c = sum(s.plugin.number_of_grids_one_dimension ** 2 for s in scs) + extra.plugin.number_of_grids_one_dimension ** 2
    with Batch([s.plugin for s in scs], capacity_agents=cap_a, capacity_cells=cap_c, capacity_scenes=6) as b:
        for i, s in enumerate(scs):
            b.set_state(i, s.pos_scale, s.vfme)
        active = {i: 0 for i in range(5)}
        b.step(3)
        for i in range(5):
            active[i] += 3
        b.set_active(1, False)
        b.set_active(3, False)
        b.step(4)
        for i in (0, 2, 4):
            active[i] += 4
        e = b.add_scene(extra.plugin)
        b.set_state(e, extra.pos_scale, extra.vfme)
        b.set_active(1, True)
        b.step(5)
        for i in (0, 1, 2, 4):
            active[i] += 5
        active[e] = 5
        b.sync()
        allsc = scs + [extra]
        for i, f in active.items():
            assert b.time(i) == f
            assert_same(b, i, alone(allsc[i], f), f"scene {i} ({f} frames)")
        with pytest.raises(MbError):
            b.add_scene(extra.plugin)  # no room left


def test_batch_many_tiny_scenes_share_tiles(built_lib, cuda):
    scs = mixed_scenes(40, seed=4, n_min=3, n_max=300)
    with Batch([s.plugin for s in scs]) as b:
        for i, s in enumerate(scs):
            b.set_state(i, s.pos_scale, s.vfme)
        b.step(8)
        for i, s in enumerate(scs):
            assert_same(b, i, alone(s, 8), f"tiny scene {i}")


def test_server_results_match_alone(built_lib, cuda):
    scs = mixed_scenes(6, seed=5, n_min=500, n_max=40_000)
    rng = np.random.default_rng(6)
    with Server(budget_bytes=2 << 30, max_scenes=16) as srv:
        handles, reqs = [], []
        owed = {}
        for s in scs:
            h, r = srv.create(s.plugin, s.pos_scale, s.vfme)
            handles.append(h)
            reqs.append(r)
            owed[h] = 1
        for _ in range(20):  # interleaved advances, submitted while frames run
            h = int(rng.choice(handles))
            k = int(rng.integers(1, 9))
            reqs.append(srv.advance(h, k))
            owed[h] += k
        lats = [srv.wait(r) for r in reqs]
        assert all(l >= 0 for l in lats)
        for h, s in zip(handles, scs):
            p, q = srv.get_state(h)
            rp, rq, _ = alone(s, owed[h])
            np.testing.assert_array_equal(p.view(np.uint32), rp.view(np.uint32), err_msg=f"scene {h}")
            np.testing.assert_array_equal(q, rq, err_msg=f"scene {h}")
        st = srv.stats()
        assert st.requests_done == len(reqs) and st.scenes == len(scs)


def test_server_rejects_over_budget(built_lib, cuda):
    big = scenes.plain_uniform(60_000, 256, seed=7)
    small = scenes.plain_uniform(1000, 32, seed=8)
    with Server(budget_bytes=64 << 20, max_scenes=4, max_agents=50_000, max_cells=100_000) as srv:
        h_small, r1 = srv.create(small.plugin, small.pos_scale, small.vfme)
        h_big, r2 = srv.create(big.plugin, big.pos_scale, big.vfme)
        srv.wait(r1)
        with pytest.raises(MbError) as e:
            srv.wait(r2)
        assert e.value.status == 5  # MB_ERR_BUDGET_EXCEEDED
        with pytest.raises(MbError):
            srv.wait(srv.advance(h_big, 3))
        srv.wait(srv.advance(h_small, 4))
        p, _ = srv.get_state(h_small)
        rp, _, _ = alone(small, 5)
        np.testing.assert_array_equal(p.view(np.uint32), rp.view(np.uint32))


def test_server_with_budget_beyond_the_key_space(built_lib, cuda):
    """A budget large enough for more than 2^28 spheres is capped to the key space
    (spheres and cells, with each scene's tile padding) instead of failing."""
    sc = scenes.plain_uniform(3000, 64, seed=21)
    with Server(budget_bytes=40 << 30, max_scenes=64) as srv:
        h, r = srv.create(sc.plugin, sc.pos_scale, sc.vfme)
        srv.wait(r)
        srv.wait(srv.advance(h, 5))
        p, _ = srv.get_state(h)
        rp, _, _ = alone(sc, 6)
        np.testing.assert_array_equal(p.view(np.uint32), rp.view(np.uint32))


def test_batch_long_steps_chain_frames(built_lib, cuda):
    """Multi-frame steps run as chains of frames in one launch while no scene
    changes mode; a held scene stays put through them."""
    scs = mixed_scenes(4, seed=31)
    with Batch([s.plugin for s in scs]) as b:
        for i, s in enumerate(scs):
            b.set_state(i, s.pos_scale, s.vfme)
        b.step(2)
        b.set_active(2, False)
        b.step(19)  # 8 + 8 + 1 + 1 + 1 frames
        b.set_active(2, True)
        b.step(9)
        b.sync()
        frames = {0: 30, 1: 30, 2: 11, 3: 30}
        for i, s in enumerate(scs):
            assert b.time(i) == frames[i]
            assert_same(b, i, alone(s, frames[i]), f"scene {i}")


@pytest.mark.parametrize("tile,fpl", [(64, 1), (256, 16), (64, 8)])
def test_batch_tuning_keeps_results(built_lib, cuda, tile, fpl):
    """A pool with other physics tiles and chain lengths gives each scene exactly
    its lone-world result."""
    scs = mixed_scenes(7, seed=21)
    with Batch([s.plugin for s in scs]) as b:
        b.set_tuning(frames_per_launch=fpl, collide_block=tile)
        for i, s in enumerate(scs):
            b.set_state(i, s.pos_scale, s.vfme)
        b.step(37)
        for i, s in enumerate(scs):
            assert_same(b, i, alone(s, 37), f"scene {i}, tile {tile}, {fpl} frames per launch")
        with pytest.raises(MbError):
            b.set_tuning(collide_block=100)


@pytest.mark.parametrize("agents", [2, 4])
def test_batch_scatter_agents(built_lib, cuda, agents):
    """2 or 4 spheres per scatter thread in a pool (the counting sort, whose scatter
    they apply to): each scene exactly its lone-world result."""
    scs = mixed_scenes(7, seed=23)
    with Batch([s.plugin for s in scs]) as b:
        b.set_tuning(scatter_agents=agents, sort_algorithm=_abi.MB_SORT_COUNTING)
        for i, s in enumerate(scs):
            b.set_state(i, s.pos_scale, s.vfme)
        b.step(19)
        for i, s in enumerate(scs):
            assert_same(b, i, alone(s, 19), f"scene {i}, {agents} spheres per scatter thread")
        with pytest.raises(MbError):
            b.set_tuning(scatter_agents=3)


def test_batch_autotune_restores_the_pool(built_lib, cuda):
    """mb_batch_autotune times its candidates on the pool and restores every
    scene (state, parity, time): the pool then continues exactly like lone worlds."""
    scs = mixed_scenes(8, seed=22)
    with Batch([s.plugin for s in scs]) as b:
        for i, s in enumerate(scs):
            b.set_state(i, s.pos_scale, s.vfme)
        b.step(5)
        res = b.autotune(frames=8)
        assert len(res["candidates"]) == _abi.MB_BATCH_TUNE_CANDIDATES
        assert all(c["ms_per_frame"] > 0 for c in res["candidates"])
        t = b.tuning
        assert {"sort_algorithm": t.sort_algorithm, "frames_per_launch": t.frames_per_launch,
                "collide_block": t.collide_block, "scatter_agents": max(t.scatter_agents, 1)} == res["best"]
        assert all(b.time(i) == 5 for i in range(len(scs)))
        b.step(20)
        for i, s in enumerate(scs):
            assert_same(b, i, alone(s, 25), f"scene {i} after autotune")
