"""CPU tests of the oracle: pinned against the reference's known-answer test and
the independent Python restatement's golden fixtures; analytic known answers."""

import math

import numpy as np
import pytest

import oracle
from bevy_millions_ball_gb300._abi import MbSettings
from tests.conftest import GOLDEN


def settings_from_fixture(d) -> MbSettings:
    s = MbSettings()
    s.max_number_of_agents = d["pos0"].shape[0]
    s.number_of_grids_one_dimension = int(d["cfg_N"])
    s.grid_size = int(d["cfg_grid_size"])
    s.half_map_height = int(d["cfg_half_map_height"])
    for i, g in enumerate(d["cfg_gravity"]):
        s.gravity[i] = float(g)
    s.e_envir, s.e_agent = float(d["cfg_e_envir"]), float(d["cfg_e_agent"])
    s.k_agent, s.c_agent, s.r_agent = float(d["cfg_k_agent"]), float(d["cfg_c_agent"]), float(d["cfg_r_agent"])
    s.time_delta = float(d["cfg_time_delta"])
    s.enable_simulation = 1
    s.enable_spring = int(d["cfg_enable_spring"])
    return s


# ------------------------------------------------------------------ hashing KAT
@pytest.mark.parametrize("n", [1, 100, 256, 16_777_216])
@pytest.mark.parametrize("passes", [3, 4])
def test_hashing_kat(n, passes):
    """src/physics/spatial_hashing.rs:536-632 (keys v mod 256, vals iota, 3 or 4 passes)."""
    if n == 16_777_216 and passes == 4:
        pytest.skip("one 16M case is enough on CPU")
    kat = np.load(GOLDEN / "hashing_kat.npz")
    keys = (np.arange(n, dtype=np.uint64) % 256).astype(np.uint32)
    sk, sv = oracle.radix_sort(keys, np.arange(n, dtype=np.uint32), passes=passes)
    start, close = oracle.spatial_hash(sk, 256)
    m = min(n, 256)
    np.testing.assert_array_equal(start[:m], kat[f"start_{n}"])
    np.testing.assert_array_equal(close[:m], kat[f"close_{n}"])
    if n > 1:
        assert np.all(np.diff(sk.astype(np.int64)) >= 0)


def test_sort_is_stable_and_matches_numpy():
    rng = np.random.default_rng(7)
    for n, cells in [(0, 1), (1, 1), (1000, 7), (100_000, 1 << 20), (300_001, 4096)]:
        keys = rng.integers(0, cells, n, dtype=np.uint32)
        passes = max(1, math.ceil(max(1, (cells - 1).bit_length()) / 8))
        sk, perm = oracle.radix_sort(keys, None, passes=passes)
        ref = np.argsort(keys, kind="stable").astype(np.uint32)
        np.testing.assert_array_equal(perm, ref)
        np.testing.assert_array_equal(sk, keys[ref])


def test_spatial_hash_empty_cells_invalid():
    sk = np.array([0, 0, 3, 3, 3, 7], np.uint32)
    start, close = oracle.spatial_hash(sk, 9)
    inv = 0xFFFFFFFF
    assert list(start) == [0, inv, inv, 2, inv, inv, inv, 5, inv]
    assert list(close) == [1, inv, inv, 4, inv, inv, inv, 5, inv]


# ------------------------------------------------------------------ physics golden
@pytest.mark.parametrize("name", ["rigid", "spring", "rigid_sparse"])
def test_oracle_matches_python_restatement(name):
    d = np.load(GOLDEN / f"physics_{name}.npz")
    w = oracle.OracleWorld(settings_from_fixture(d))
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
        full = d[f"f{f}_start"] != 0xFFFFFFFF
        np.testing.assert_array_equal(dbg["close"][full], d[f"f{f}_close"][full])


def test_fixtures_exercise_contacts_walls_and_jitter():
    """The golden scenes must actually hit the branches they are meant to pin."""
    d = np.load(GOLDEN / "physics_rigid.npz")
    p0 = d["f1_pos"]
    r = p0[:, 3]
    # wall contact: somebody sits exactly on a clamped face
    H = float(d["cfg_half_map_height"])
    assert np.any(np.isclose(p0[:, 1], r)) or np.any(np.isclose(p0[:, 1], 2 * H - r))
    # agent contacts: velocities differ from pure free fall for many agents
    from bevy_millions_ball_gb300 import unpack_vfme

    v0, _, _ = unpack_vfme(d["f0_vfme"])
    v1, _, _ = unpack_vfme(d["f1_vfme"])
    assert np.mean(np.abs(v1[:, 0] - v0[d["f1_perm"], 0]) > 1e-4) > 0.05


# ------------------------------------------------------------------ f16 packing
def test_f16_rne_matches_numpy():
    L = oracle.lib()
    rng = np.random.default_rng(3)
    vals = np.concatenate([
        rng.standard_normal(20000).astype(np.float32) * np.float32(10.0),
        (rng.standard_normal(5000) * 1e-5).astype(np.float32),   # f16 subnormals
        (rng.standard_normal(2000) * 1e-8).astype(np.float32),   # underflow
        np.array([0.0, -0.0, 65504.0, 65519.99, 65520.0, -65520.0, 2.0**-24, 2.0**-25, 3 * 2.0**-26,
                  1.0009765625, 1.00048828125, 1.00146484375], np.float32),
    ])
    ours = np.array([L.mbo_f32_to_f16(float(v)) for v in vals], np.uint16)
    ref = vals.astype(np.float16).view(np.uint16)
    np.testing.assert_array_equal(ours, ref)
    back = np.array([L.mbo_f16_to_f32(int(h)) for h in ref[:3000]], np.float32)
    np.testing.assert_array_equal(back, ref[:3000].view(np.float16).astype(np.float32))


def test_hash3f1u():
    L = oracle.lib()
    import ctypes as C

    out = (C.c_float * 3)()
    for n in [0, 1, 2, 12345, 65535, 1 << 20, 0xFFFFFFFF]:
        L.mbo_hash3f1u(n, out)
        v = (n * (n ^ (n >> 15))) & 0xFFFFFFFF
        exp = [np.float32(np.float32((v * m) & 0xFFFFFFFF) / np.float32(2.0**32)) for m in (1, 0x1FF, 0x3FFFF)]
        assert list(out) == exp


# ------------------------------------------------------------------ analytic KATs
def one_sphere(pos, vel, H=8, N=4, g=(0.0, -9.81, 0.0), e=0.8, spring=False, k=25.0, c=0.1, dt=1 / 60):
    s = MbSettings()
    s.max_number_of_agents = len(pos)
    s.number_of_grids_one_dimension = N
    s.grid_size = 4
    s.half_map_height = H
    for i in range(3):
        s.gravity[i] = g[i]
    s.e_envir = s.e_agent = e
    s.k_agent, s.c_agent, s.r_agent = k, c, 0.9
    s.time_delta = dt
    s.enable_simulation = 1
    s.enable_spring = 1 if spring else 0
    from bevy_millions_ball_gb300 import pack_vfme

    w = oracle.OracleWorld(s, threads=1)
    p = np.asarray(pos, np.float32)
    w.set_state(p, pack_vfme(np.asarray(vel, np.float32), np.zeros((len(pos), 3), np.float32), 1.0))
    return w


def test_free_fall_closed_form():
    """v_{t+1} = v_t + g dt^2 (f16 stored), p_{t+1} = p_t + v_{t+1}; dt quantised to 0.016."""
    w = one_sphere([[0.0, 12.0, 0.0, 0.5]], [[0.0, 0.0, 0.0]])
    w.step(21)  # INIT + 20 LOOP frames
    dt = np.float32(0.016)
    g = np.float32(-9.81)
    p, q = w.get_state()
    # independent recurrence: velocity is re-rounded to f16 every frame
    v = np.float32(0.0)
    y = np.float32(12.0)
    for _ in range(20):
        vv = np.float32(v + np.float32(np.float32(g * dt) * dt))
        y = np.float32(y + vv)
        v = np.float32(np.float16(vv))
    assert p[0, 1] == y
    from bevy_millions_ball_gb300 import unpack_vfme

    assert unpack_vfme(q)[0][0, 1] == v


def test_floor_bounce_restitution():
    """Rigid wall: position clamped to r, velocity component times -e (physics.wgsl:278-280)."""
    w = one_sphere([[0.0, 0.55, 0.0, 0.5]], [[0.0, -0.2, 0.0]], g=(0.0, 0.0, 0.0))
    w.step(2)
    p, q = w.get_state()
    from bevy_millions_ball_gb300 import unpack_vfme

    assert p[0, 1] == np.float32(0.5)
    v16 = np.float32(np.float16(-0.2))
    expected = np.float32(np.float16(np.float32(v16 * np.float32(-0.8))))
    assert unpack_vfme(q)[0][0, 1] == expected


def test_head_on_collision_rigid():
    """Two equal spheres approaching along x: rigid response exchanges momentum scaled by e."""
    w = one_sphere([[-0.45, 4.0, 0.0, 0.5], [0.45, 4.0, 0.0, 0.5]], [[0.05, 0.0, 0.0], [-0.05, 0.0, 0.0]],
                   g=(0.0, 0.0, 0.0))
    w.step(2)
    p, q = w.get_state()
    from bevy_millions_ball_gb300 import unpack_vfme

    v = unpack_vfme(q)[0]
    # each sphere ends moving away from the other (e = 0.8), symmetric
    xs = p[:, 0]
    left, right = np.argmin(xs), np.argmax(xs)
    assert v[left, 0] < 0 < v[right, 0]
    assert abs(abs(v[left, 0]) - 0.8 * 0.05) < 2e-3
    assert xs[right] - xs[left] > 0.9


def test_spring_wall_force_sign():
    """Spring wall: Hooke force pushes back inside (physics.wgsl:282-286)."""
    w = one_sphere([[0.0, 0.45, 0.0, 0.5]], [[0.0, 0.0, 0.0]], g=(0.0, 0.0, 0.0), spring=True, k=100.0, c=0.0)
    w.step(2)
    _, q = w.get_state()
    from bevy_millions_ball_gb300 import unpack_vfme

    f = unpack_vfme(q)[1]
    assert f[0, 1] > 0  # floor at y=0 pushes up


def test_reference_default_lattice():
    """src/physics/mod.rs:172-212: 2^(L//2) x 2^(L - L//2) lattice, x-major, spacing 4."""
    from bevy_millions_ball_gb300 import PhysicsPlugin, scenes, unpack_vfme
    sc = scenes.reference_default(PhysicsPlugin(max_number_of_agents=1 << 13))
    p = sc.pos_scale
    assert p.shape == (8192, 4)
    # count_x = 2^6 = 64 rows of count_z = 2^7 = 128
    assert p[0, 0] == -0.5 * 63 * 4 and p[0, 2] == -0.5 * 127 * 4
    assert p[127, 0] == p[0, 0] and p[127, 2] == 0.5 * 127 * 4
    assert p[128, 0] == p[0, 0] + 4 and p[128, 2] == p[0, 2]
    assert np.all(p[:, 1] == 4.0) and np.all(p[:, 3] == 1.0)
    v, f, m = unpack_vfme(sc.vfme)
    assert np.all(np.abs(v[:, [0, 2]]) <= 0.8) and np.all(v[:, 1] == 0) and np.all(f == 0) and np.all(m == 1)
    with pytest.raises(ValueError):
        scenes.reference_default(PhysicsPlugin(max_number_of_agents=1000))
