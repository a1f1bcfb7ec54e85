"""GPU parity of whole frames (sort -> cell ranges -> physics) through the C ABI,
against the oracle and the golden fixtures.

Bar: keys, permutation and cell ranges bit-exact; positions and packed velocity /
force bit-exact as well (the physics kernel rounds like the oracle).  The stated
float tolerances (|dx| <= 1e-5 after 1 frame, <= 1e-3 after 10 frames) are also
asserted explicitly, although bit-exactness implies them.
"""

import numpy as np
import pytest

import oracle
from bevy_millions_ball_gb300 import MbError, PhysicsPlugin, World, _abi, pack_vfme, scenes
from tests.conftest import GOLDEN
from tests.test_oracle import settings_from_fixture

pytestmark = pytest.mark.gpu
INV = 0xFFFFFFFF
TOL_1 = 1e-5   # position error after 1 frame
TOL_10 = 1e-3  # position error after 10 frames


def plugin_from_settings(s) -> PhysicsPlugin:
    return PhysicsPlugin.from_c(s)


def compare(world: World, ow: "oracle.OracleWorld", frame: int, tol: float | None = None):
    p, q = world.get_state()
    rp, rq = ow.get_state()
    d, rd = world.debug(), ow.debug()
    np.testing.assert_array_equal(d["keys"], rd["keys"], err_msg=f"keys, frame {frame}")
    np.testing.assert_array_equal(d["perm"], rd["perm"], err_msg=f"perm, frame {frame}")
    np.testing.assert_array_equal(d["start"], rd["start"], err_msg=f"start, frame {frame}")
    full = rd["start"] != INV
    np.testing.assert_array_equal(d["close"][full], rd["close"][full], err_msg=f"close, frame {frame}")
    if tol is not None:
        assert np.nanmax(np.abs(p[:, :3] - rp[:, :3])) <= tol
    np.testing.assert_array_equal(p.view(np.uint32), rp.view(np.uint32), err_msg=f"pos, frame {frame}")
    np.testing.assert_array_equal(q, rq, err_msg=f"vfme, frame {frame}")


@pytest.mark.parametrize("name", ["rigid", "spring", "rigid_sparse"])
def test_world_matches_golden_fixtures(built_lib, cuda, name):
    d = np.load(GOLDEN / f"physics_{name}.npz")
    with World(plugin_from_settings(settings_from_fixture(d))) as w:
        w.set_state(d["pos0"], d["vfme0"])
        for f in range(int(d["frames"])):
            w.step(1)
            p, q = w.get_state()
            dbg = w.debug()
            np.testing.assert_array_equal(p.view(np.uint32), d[f"f{f}_pos"].view(np.uint32), err_msg=f"frame {f}")
            np.testing.assert_array_equal(q, d[f"f{f}_vfme"])
            np.testing.assert_array_equal(dbg["keys"], d[f"f{f}_keys"])
            np.testing.assert_array_equal(dbg["perm"], d[f"f{f}_perm"])
            np.testing.assert_array_equal(dbg["start"], d[f"f{f}_start"])


def run_pair(scene, frames, checkpoints, world_kw=None, tuning=None):
    with World(scene.plugin, **(world_kw or {})) as w:
        if tuning:
            w.set_tuning(**tuning)
        ow = oracle.OracleWorld(scene.plugin.to_c())
        w.set_state(scene.pos_scale, scene.vfme)
        ow.set_state(scene.pos_scale, scene.vfme)
        done = 0
        for cp in checkpoints:
            w.step(cp - done)
            ow.step(cp - done)
            done = cp
            w.sync()
            tol = TOL_1 if cp == 2 else (TOL_10 if cp == 11 else None)
            compare(w, ow, cp, tol)
        assert w.time == ow.time == done


def test_small_uniform_rigid(built_lib, cuda):
    """65,536 spheres, N=256 (the small plain workload), 100 frames."""
    sc = scenes.workload("P-small")
    run_pair(sc, 101, [1, 2, 11, 50, 101])


def test_uniform_spring(built_lib, cuda):
    sc = scenes.plain_uniform(50_000, 256, seed=4, spring=True, k=400.0, c=4.0)
    run_pair(sc, 60, [1, 2, 11, 60])


def test_clustered_spring(built_lib, cuda):
    """Uneven occupancy (~40 spheres per cell at cluster centres)."""
    sc = scenes.plain_clustered(262_144, 512, clusters=4, sigma_xz=16.0, seed=9)
    run_pair(sc, 40, [1, 2, 11, 40])


@pytest.mark.parametrize("spring", [False, True])
def test_mixed_masses_and_radii(built_lib, cuda, spring):
    """Masses whose sums are powers of two (den = m1 + m2 in 2, 4, ...) and ones
    that are not, radii 0.3-0.6: both ways the contact solve divides stay exact."""
    sc = scenes.plain_uniform(40_000, 128, half_map_height=4, seed=31, spring=spring)
    rng = np.random.default_rng(32)
    from bevy_millions_ball_gb300 import unpack_vfme
    v, f, _ = unpack_vfme(sc.vfme)
    mass = rng.choice(np.array([0.5, 1.0, 1.5, 2.0, 3.0, 0.7, 1.25], np.float32), sc.n)
    sc.vfme = pack_vfme(v, f, mass)
    sc.pos_scale[:, 3] = rng.choice(np.array([0.3, 0.45, 0.5, 0.6], np.float32), sc.n)
    run_pair(sc, 40, [1, 2, 11, 40])


def test_nonpow2_grid_and_grid_size(built_lib, cuda):
    sc = scenes.plain_uniform(30_000, 300, grid_size=2, half_map_height=4, seed=12)
    run_pair(sc, 30, [1, 2, 11, 30])


@pytest.mark.parametrize("grid_size", [3, 7])
def test_odd_grid_sizes(built_lib, cuda, grid_size):
    """Cell index = u32(x + H_s) / grid_size for divisors that are not powers of two."""
    sc = scenes.plain_uniform(20_000, 64, grid_size=grid_size, half_map_height=4, seed=40 + grid_size)
    run_pair(sc, 12, [1, 2, 12])


def test_sparse_grid_more_cells_than_agents(built_lib, cuda):
    """C = N*N > n: every cell cleared, not just n (the reference needs n >= N*N)."""
    sc = scenes.plain_uniform(5_000, 512, seed=13)
    run_pair(sc, 25, [1, 2, 11, 25])


@pytest.mark.parametrize("digit_bits", [4, 6, 8, 11])
def test_onesweep_digit_widths_agree(built_lib, cuda, digit_bits):
    """The world with the onesweep radix sort instead of the counting sort."""
    sc = scenes.plain_uniform(70_000, 256, seed=21)
    with World(sc.plugin) as w:
        w.set_tuning(digit_bits_max=digit_bits, sort_algorithm=1)
        ow = oracle.OracleWorld(sc.plugin.to_c())
        w.set_state(sc.pos_scale, sc.vfme)
        ow.set_state(sc.pos_scale, sc.vfme)
        w.step(12)
        ow.step(12)
        compare(w, ow, 12)


def test_switch_sort_algorithm_midrun(built_lib, cuda):
    """Counting <-> onesweep switches keep the frame sequence identical."""
    sc = scenes.plain_clustered(120_000, 256, clusters=3, sigma_xz=12.0, seed=17)
    with World(sc.plugin) as w:
        ow = oracle.OracleWorld(sc.plugin.to_c())
        w.set_state(sc.pos_scale, sc.vfme)
        ow.set_state(sc.pos_scale, sc.vfme)
        for alg, k in [(1, 3), (0, 4), (1, 2), (0, 5)]:
            w.set_tuning(sort_algorithm=alg)
            w.step(k)
            ow.step(k)
            compare(w, ow, ow.time)
    with World(sc.plugin) as w:  # onesweep from the upload on
        w.set_tuning(sort_algorithm=1)
        ow = oracle.OracleWorld(sc.plugin.to_c())
        w.set_state(sc.pos_scale, sc.vfme)
        ow.set_state(sc.pos_scale, sc.vfme)
        w.step(6)
        ow.step(6)
        compare(w, ow, 6)


def test_settings_change_midrun(built_lib, cuda):
    """Runtime edits (the egui path) including a grid change that re-keys the agents."""
    sc = scenes.plain_uniform(40_000, 256, seed=3)
    with World(sc.plugin) as w:
        ow = oracle.OracleWorld(sc.plugin.to_c())
        w.set_state(sc.pos_scale, sc.vfme)
        ow.set_state(sc.pos_scale, sc.vfme)
        w.step(5)
        ow.step(5)
        for new in [sc.plugin.replace(e_agent=0.3, gravity=(0.5, -3.0, 0.0)),
                    sc.plugin.replace(enable_spring=True, k_agent=300.0, c_agent=2.0),
                    sc.plugin.replace(number_of_grids_one_dimension=128, grid_size=2),
                    sc.plugin.replace(number_of_grids_one_dimension=512, grid_size=1)]:
            w.set_settings(new)
            ow.set_settings(new.to_c())
            w.step(4)
            ow.step(4)
            compare(w, ow, ow.time)


def test_crowded_cells_block_sort(built_lib, cuda):
    """~200 spheres per cell: cells put back in input order by the warp bitonic
    fixup path (9-256 slots); the crowded-warp contact walk (six candidates per step)."""
    sc = scenes.plain_uniform(51_200, 16, grid_size=1, half_map_height=8, seed=31)
    run_pair(sc, 4, [1, 2, 4])


def test_degenerate_cells_heapsort(built_lib, cuda):
    """~9,000 spheres per cell (N=2): the block fixup path (bitmaps of the input
    indices, cells over 256 slots) and bands too wide to stage (global reads)."""
    sc = scenes.plain_uniform(36_000, 2, grid_size=4, half_map_height=8, seed=32)
    run_pair(sc, 3, [1, 2, 3])


INDIRECT = {"state_gather": 1}


@pytest.mark.parametrize("case", ["small", "clustered", "crowded", "degenerate", "mixed", "sparse"])
def test_indirect_state_gather(built_lib, cuda, case):
    """MB_GATHER_INDIRECT: the sort writes only the permutation and the physics
    pass gathers its bands and spheres through it (staged bands, and the global
    reads of bands too wide to stage); bit-exact like the sorted-copy mode."""
    if case == "small":
        run_pair(scenes.workload("P-small"), 101, [1, 2, 11, 50, 101], tuning=INDIRECT)
    elif case == "clustered":
        run_pair(scenes.plain_clustered(262_144, 512, clusters=4, sigma_xz=16.0, seed=9), 40, [1, 2, 11, 40],
                 tuning=INDIRECT)
    elif case == "crowded":
        run_pair(scenes.plain_uniform(51_200, 16, grid_size=1, half_map_height=8, seed=31), 4, [1, 2, 4],
                 tuning=INDIRECT)
    elif case == "degenerate":
        run_pair(scenes.plain_uniform(36_000, 2, grid_size=4, half_map_height=8, seed=32), 3, [1, 2, 3],
                 tuning=INDIRECT)
    elif case == "mixed":
        sc = scenes.plain_uniform(40_000, 128, half_map_height=4, seed=31, spring=True)
        rng = np.random.default_rng(33)
        from bevy_millions_ball_gb300 import unpack_vfme
        v, f, _ = unpack_vfme(sc.vfme)
        sc.vfme = pack_vfme(v, f, rng.choice(np.array([0.5, 1.0, 1.5, 2.0, 0.7], np.float32), sc.n))
        sc.pos_scale[:, 3] = rng.choice(np.array([0.3, 0.45, 0.5, 0.6], np.float32), sc.n)
        run_pair(sc, 30, [1, 2, 11, 30], tuning=INDIRECT)
    else:
        run_pair(scenes.plain_uniform(5_000, 512, seed=13), 25, [1, 2, 11, 25], tuning=INDIRECT)


def test_indirect_with_onesweep_and_switches(built_lib, cuda):
    """The gather mode with the onesweep sort, and switched mid-run both ways."""
    sc = scenes.plain_clustered(120_000, 256, clusters=3, sigma_xz=12.0, seed=18)
    with World(sc.plugin) as w:
        ow = oracle.OracleWorld(sc.plugin.to_c())
        w.set_state(sc.pos_scale, sc.vfme)
        ow.set_state(sc.pos_scale, sc.vfme)
        for alg, gather, k in [(1, 1, 3), (0, 1, 4), (0, 0, 2), (1, 0, 2), (0, 1, 5)]:
            w.set_tuning(sort_algorithm=alg, state_gather=gather)
            w.step(k)
            ow.step(k)
            compare(w, ow, ow.time)
        with pytest.raises(MbError):
            w.set_tuning(state_gather=2)


@pytest.mark.parametrize("tile", [64, 256])
@pytest.mark.parametrize("case", ["small", "clustered", "crowded", "degenerate", "sparse"])
def test_collide_block_sizes(built_lib, cuda, case, tile):
    """Physics tiles of 64 and 256 slots per thread block (collide_block), with
    the sorted copy and with the gather through the permutation: bit-exact."""
    for gather in (0, 1):
        tuning = {"collide_block": tile, "state_gather": gather}
        if case == "small":
            run_pair(scenes.workload("P-small"), 51, [1, 2, 11, 51], tuning=tuning)
        elif case == "clustered":
            run_pair(scenes.plain_clustered(262_144, 512, clusters=4, sigma_xz=16.0, seed=9), 20, [1, 2, 20],
                     tuning=tuning)
        elif case == "crowded":
            run_pair(scenes.plain_uniform(51_200, 16, grid_size=1, half_map_height=8, seed=31), 4, [1, 2, 4],
                     tuning=tuning)
        elif case == "degenerate":
            run_pair(scenes.plain_uniform(36_000, 2, grid_size=4, half_map_height=8, seed=32), 3, [1, 2, 3],
                     tuning=tuning)
        else:
            run_pair(scenes.plain_uniform(5_000 + tile, 512, seed=13), 25, [1, 2, 25], tuning=tuning)
    with World(scenes.plain_uniform(1000, 32).plugin) as w:
        with pytest.raises(MbError):
            w.set_tuning(collide_block=96)


@pytest.mark.parametrize("agents", [2, 4])
@pytest.mark.parametrize("case", ["small", "clustered", "crowded", "ragged"])
def test_scatter_agents(built_lib, cuda, case, agents):
    """scatter_agents: 2 or 4 spheres per thread of the counting sort's scatter
    (grid-stride steps of 256 x agents inputs, ragged tails); bit-exact against
    the oracle, with the sorted copy and with the gather through the permutation."""
    for gather in (0, 1):
        tuning = {"scatter_agents": agents, "state_gather": gather}
        if case == "small":
            run_pair(scenes.workload("P-small"), 21, [1, 2, 21], tuning=tuning)
        elif case == "clustered":
            run_pair(scenes.plain_clustered(262_144, 512, clusters=4, sigma_xz=16.0, seed=9), 12, [1, 2, 12],
                     tuning=tuning)
        elif case == "crowded":
            run_pair(scenes.plain_uniform(51_200, 16, grid_size=1, half_map_height=8, seed=31), 4, [1, 2, 4],
                     tuning=tuning)
        else:  # n not a multiple of the step, smaller than one block's step
            run_pair(scenes.plain_uniform(777 + 256 * agents + 3, 64, seed=14), 25, [1, 2, 25], tuning=tuning)
    with World(scenes.plain_uniform(1000, 32).plugin) as w:
        for bad in (3, 5, 8):
            with pytest.raises(MbError):
                w.set_tuning(scatter_agents=bad)


FUSED = {"frame_kernel": 1, "sort_algorithm": 0}  # fused frames run the claim-and-fixup counting sort


@pytest.mark.parametrize("gather", [0, 1])
@pytest.mark.parametrize("case", ["small", "clustered", "crowded", "degenerate", "sparse", "mixed"])
def test_fused_frame_kernel(built_lib, cuda, case, gather):
    """MB_FRAME_FUSED: every stage of every frame of a step in one cooperative
    kernel (grid barriers between the stages); bit-exact like the per-stage
    kernels, with the sorted copy and with the gather through the permutation."""
    tuning = dict(FUSED, state_gather=gather)
    if case == "small":
        run_pair(scenes.workload("P-small"), 101, [1, 2, 11, 50, 101], tuning=tuning)
    elif case == "clustered":
        run_pair(scenes.plain_clustered(262_144, 512, clusters=4, sigma_xz=16.0, seed=9), 40, [1, 2, 11, 40],
                 tuning=tuning)
    elif case == "crowded":
        run_pair(scenes.plain_uniform(51_200, 16, grid_size=1, half_map_height=8, seed=31), 4, [1, 2, 4],
                 tuning=tuning)
    elif case == "degenerate":
        run_pair(scenes.plain_uniform(36_000, 2, grid_size=4, half_map_height=8, seed=32), 3, [1, 2, 3],
                 tuning=tuning)
    elif case == "sparse":
        run_pair(scenes.plain_uniform(5_000, 512, seed=13), 25, [1, 2, 11, 25], tuning=tuning)
    else:
        sc = scenes.plain_uniform(40_000, 128, half_map_height=4, seed=34, spring=True)
        rng = np.random.default_rng(35)
        from bevy_millions_ball_gb300 import unpack_vfme
        v, f, _ = unpack_vfme(sc.vfme)
        sc.vfme = pack_vfme(v, f, rng.choice(np.array([0.5, 1.0, 1.5, 2.0, 0.7], np.float32), sc.n))
        sc.pos_scale[:, 3] = rng.choice(np.array([0.3, 0.45, 0.5, 0.6], np.float32), sc.n)
        run_pair(sc, 30, [1, 2, 11, 30], tuning=tuning)


def test_fused_switches_and_settings(built_lib, cuda):
    """Fused and per-stage frames alternate mid-run (odd and even frame counts per
    step, so both state buffers start fused launches), with a settings change
    and a re-upload in between; the sort algorithm must stay counting."""
    sc = scenes.plain_uniform(60_000, 256, seed=44)
    with World(sc.plugin) as w:
        ow = oracle.OracleWorld(sc.plugin.to_c())
        w.set_state(sc.pos_scale, sc.vfme)
        ow.set_state(sc.pos_scale, sc.vfme)
        for kernel, k in [(1, 1), (1, 3), (0, 2), (1, 7), (0, 5), (1, 16)]:
            w.set_tuning(frame_kernel=kernel, sort_algorithm=0)
            w.step(k)
            ow.step(k)
            w.sync()
            compare(w, ow, ow.time)
        new = sc.plugin.replace(e_agent=0.4, number_of_grids_one_dimension=128, grid_size=2)
        w.set_settings(new)
        ow.set_settings(new.to_c())
        w.step(9)
        ow.step(9)
        compare(w, ow, ow.time)
        w.set_state(sc.pos_scale, sc.vfme)
        ow.set_state(sc.pos_scale, sc.vfme)
        w.step(12)
        ow.step(12)
        compare(w, ow, ow.time)
        with pytest.raises(MbError):
            w.set_tuning(sort_algorithm=1)  # fused frames run the counting sort
        with pytest.raises(MbError):
            w.set_tuning(frame_kernel=2)


def test_full_size_1m_properties(built_lib, cuda):
    """Size-independent properties after many frames at full size."""
    sc = scenes.workload("P-1M")
    with World(sc.plugin) as w:
        w.set_state(sc.pos_scale, sc.vfme)
        w.step(200)
        w.sync()
        p, q = w.get_state()
        d = w.debug()
        n = sc.n
        assert np.array_equal(np.sort(d["perm"]), np.arange(n, dtype=np.uint32))  # a permutation
        # every cell's range is consistent and the ranges tile [0, n)
        full = d["start"] != INV
        sizes = (d["close"][full].astype(np.int64) - d["start"][full] + 1)
        assert sizes.sum() == n and np.all(sizes >= 1)
        order = np.argsort(d["start"][full])
        st = d["start"][full][order].astype(np.int64)
        assert st[0] == 0 and np.all(st[1:] == (st[:-1] + sizes[order][:-1]))
        hs = 512
        assert np.all(np.abs(p[:, 0]) <= hs) and np.all(np.abs(p[:, 2]) <= hs)
        assert np.all(p[:, 1] >= 0.5 - 1e-6) and np.all(p[:, 1] <= 15.5 + 1e-6)
        assert not np.isnan(p).any()


def check_frame_properties(w, plugin, n):
    """Size-independent properties of a world after a LOOP frame: the order is a
    stable permutation, the cell ranges tile [0, n) in cell order, and every
    emitted key is the cell of the sphere's position."""
    p, _ = w.get_state()
    d = w.debug()
    perm = d["perm"].astype(np.int64)
    assert np.array_equal(np.sort(perm), np.arange(n))  # a permutation
    full = d["start"] != INV
    cells = np.nonzero(full)[0]
    st = d["start"][full].astype(np.int64)
    sizes = d["close"][full].astype(np.int64) - st + 1
    assert sizes.sum() == n and np.all(sizes >= 1)
    assert st[0] == 0 and np.all(st[1:] == st[:-1] + sizes[:-1])  # ranges in cell order, back to back
    cell_of_slot = np.repeat(cells, sizes)
    # stable: inside a cell the old slots ascend
    same = cell_of_slot[1:] == cell_of_slot[:-1]
    assert np.all(perm[1:][same] > perm[:-1][same])
    # keys emitted for the next frame are the cells of the new positions
    N, g = plugin.number_of_grids_one_dimension, plugin.grid_size
    H = np.float32(N * g // 2)
    def cell(v):
        u = np.clip(np.trunc((v + H).astype(np.float32)), 0, 2.0**32 - 1).astype(np.uint64)
        return np.minimum(u // g, N - 1)
    keys = cell(p[:, 2]) * N + cell(p[:, 0])
    np.testing.assert_array_equal(d["keys"].astype(np.uint64), keys)
    assert not np.isnan(p).any()


def test_clustered_4m_properties(built_lib, cuda):
    """The 4,194,304-sphere clustered spring workload: stable order, cell ranges
    and keys after 20 frames (cells near the cluster centres hold ~100 spheres)."""
    sc = scenes.workload("P-4M")
    with World(sc.plugin) as w:
        w.set_state(sc.pos_scale, sc.vfme)
        w.step(20)
        w.sync()
        check_frame_properties(w, sc.plugin, sc.n)


def test_16m_uniform_properties(built_lib, cuda):
    """16,777,216 spheres on a 4096 x 4096 grid (16x the benchmark scene)."""
    sc = scenes.plain_uniform(1 << 24, 4096, seed=77)
    with World(sc.plugin) as w:
        w.set_state(sc.pos_scale, sc.vfme)
        w.step(3)
        w.sync()
        check_frame_properties(w, sc.plugin, sc.n)


def test_disabled_simulation_is_noop(built_lib, cuda):
    sc = scenes.plain_uniform(4096, 64, seed=1)
    with World(sc.plugin.replace(enable_simulation=False)) as w:
        w.set_state(sc.pos_scale, sc.vfme)
        w.step(5)
        p, q = w.get_state()
        assert w.time == 0
        np.testing.assert_array_equal(p, sc.pos_scale)


def test_reupload_restarts_with_init(built_lib, cuda):
    sc = scenes.plain_uniform(8192, 128, seed=2)
    with World(sc.plugin) as w:
        ow = oracle.OracleWorld(sc.plugin.to_c())
        w.set_state(sc.pos_scale, sc.vfme)
        w.step(7)
        w.set_state(sc.pos_scale, sc.vfme)
        ow.set_state(sc.pos_scale, sc.vfme)
        assert w.time == 0
        w.step(6)
        ow.step(6)
        compare(w, ow, 6)


def test_device_pointer_state_roundtrip(built_lib, cuda):
    torch = cuda
    sc = scenes.plain_uniform(10_000, 128, seed=6)
    dp = torch.from_numpy(sc.pos_scale.copy()).cuda()
    dq = torch.from_numpy(sc.vfme.view(np.int32).copy()).cuda()
    with World(sc.plugin, stream=torch.cuda.current_stream().cuda_stream) as w:
        w.set_state_device(dp.data_ptr(), dq.data_ptr())
        w.step(3)
        out_p = torch.empty_like(dp)
        out_q = torch.empty_like(dq)
        w.get_state_device(out_p.data_ptr(), out_q.data_ptr())
        torch.cuda.synchronize()
        p, q = w.get_state()
        np.testing.assert_array_equal(out_p.cpu().numpy(), p)
        np.testing.assert_array_equal(out_q.cpu().numpy().view(np.uint32), q)
        a, b = w.device_buffers()
        assert a and b


def test_errors_are_reported_not_fatal(built_lib, cuda):
    with pytest.raises(MbError) as e:
        World(PhysicsPlugin(number_of_grids_one_dimension=0))
    assert e.value.status == 1
    with pytest.raises(MbError):
        World(PhysicsPlugin(time_delta=0.0001))  # quantises to 0
    w = World(PhysicsPlugin(max_number_of_agents=1024, number_of_grids_one_dimension=32, grid_size=1))
    with pytest.raises(MbError) as e:
        w.step(1)  # no state yet
    assert e.value.status == 6
    with pytest.raises(MbError):
        w.set_settings(PhysicsPlugin(max_number_of_agents=2048))
    with pytest.raises(MbError):
        w.set_tuning(digit_bits_max=12)
    with pytest.raises(MbError):
        w.set_tuning(sort_algorithm=7)
    w.close()


def test_single_agent_and_tiny_grid(built_lib, cuda):
    p = PhysicsPlugin(max_number_of_agents=1, number_of_grids_one_dimension=1, grid_size=4, half_map_height=2)
    pos = np.array([[0.3, 3.0, -0.2, 0.5]], np.float32)
    q = pack_vfme(np.array([[0.01, 0.0, 0.02]], np.float32), np.zeros((1, 3), np.float32), 1.0)
    with World(p) as w:
        ow = oracle.OracleWorld(p.to_c())
        w.set_state(pos, q)
        ow.set_state(pos, q)
        w.step(30)
        ow.step(30)
        compare(w, ow, 30)


def test_autotune_keeps_the_frame_sequence(built_lib, cuda):
    """mb_autotune times its candidates on the scene and restores the saved frame:
    the world then continues exactly like the oracle that never paused."""
    sc = scenes.workload("P-small")
    with World(sc.plugin) as w:
        ow = oracle.OracleWorld(sc.plugin.to_c())
        w.set_state(sc.pos_scale, sc.vfme)
        ow.set_state(sc.pos_scale, sc.vfme)
        w.step(5)
        ow.step(5)
        res = w.autotune(frames=8)
        assert len(res["candidates"]) == _abi.MB_TUNE_CANDIDATES
        assert all(c["ms_per_frame"] > 0 for c in res["candidates"])
        fastest = min(res["candidates"], key=lambda c: c["ms_per_frame"])
        assert res["best"] == {k: fastest[k] for k in res["best"]}
        t = w.tuning
        assert (t.sort_algorithm, t.digit_bits_max, t.frames_per_launch, t.state_gather,
                t.frame_kernel, t.collide_block, max(t.scatter_agents, 1)) == tuple(res["best"].values())
        assert w.time == 5
        compare(w, ow, 5)
        w.step(21)
        ow.step(21)
        compare(w, ow, 26)


@pytest.mark.parametrize("fpl", [1, 2, 16])
def test_frames_per_launch(built_lib, cuda, fpl):
    sc = scenes.plain_uniform(30_000, 256, seed=50 + fpl)
    with World(sc.plugin) as w:
        w.set_tuning(frames_per_launch=fpl)
        ow = oracle.OracleWorld(sc.plugin.to_c())
        w.set_state(sc.pos_scale, sc.vfme)
        ow.set_state(sc.pos_scale, sc.vfme)
        w.step(37)
        ow.step(37)
        compare(w, ow, 37)
        with pytest.raises(MbError):
            w.set_tuning(frames_per_launch=3)


def test_reference_default_scene(built_lib, cuda):
    """The reference plugin's default settings and its start-up lattice (16,384
    spheres of radius 1 at spacing 4, N = 128, grid_size 8, dt = 1/120)."""
    sc = scenes.reference_default()
    run_pair(sc, 60, [1, 2, 11, 60])


def test_device_state_views(built_lib, cuda):
    """Zero-copy device views of the state buffers (torch reads them in place)."""
    torch = cuda
    sc = scenes.plain_uniform(5000, 64, seed=3)
    with World(sc.plugin) as w:
        w.set_state(sc.pos_scale, sc.vfme)
        w.step(4)
        w.sync()
        pv, qv = w.device_state()
        tp = torch.as_tensor(pv, device="cuda")
        assert tp.shape == (5000, 4) and tp.dtype == torch.float32
        assert tp.data_ptr() == w.device_buffers()[0]  # a view, not a copy
        p, q = w.get_state()
        np.testing.assert_array_equal(tp.cpu().numpy(), p)
        assert qv.__cuda_array_interface__["typestr"] == "<u4" and qv.__cuda_array_interface__["shape"] == (5000, 4)
        tq = torch.empty((5000, 4), dtype=torch.int32, device="cuda")
        scratch = torch.empty_like(tp)
        w.get_state_device(scratch.data_ptr(), tq.data_ptr())
        torch.cuda.synchronize()
        np.testing.assert_array_equal(tq.cpu().numpy().view(np.uint32), q)
