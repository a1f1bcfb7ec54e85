"""CPU tests of the C ABI: the library builds, loads and exports every declared
symbol; host-side logic (defaults, constant quantisation) matches the reference
and the oracle.  No device work is issued here."""

import ctypes as C
import math
import re

import numpy as np
import pytest

import oracle
from bevy_millions_ball_gb300 import PhysicsPlugin, PhysicsSettings, _abi, pack_vfme, scenes, unpack_vfme
from tests.conftest import ROOT


def declared_functions():
    text = (ROOT / "include" / "millionsball.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mb_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ["mb_create", "mb_destroy", "mb_set_settings", "mb_set_state", "mb_get_state", "mb_step",
                 "mb_sync", "mb_get_debug", "mb_device_buffers", "mb_sort_and_hash", "mb_last_error"]:
        assert must in names


def test_library_exports_every_declared_symbol(built_lib):
    missing = [n for n in declared_functions() if not hasattr(built_lib, n)]
    assert not missing, missing
    assert set(declared_functions()) <= set(_abi.SIGNATURES), "ctypes bindings must cover the header"
    assert b"sm_103a" in built_lib.mb_version()


def test_struct_layout():
    assert C.sizeof(_abi.MbSettings) == 56
    assert C.sizeof(_abi.MbConsts) == 56
    assert C.sizeof(_abi.MbTuning) == 32


def test_defaults_match_reference_plugin(built_lib):
    """PhysicsPlugin::default (src/physics/mod.rs:87-109)."""
    s = _abi.MbSettings()
    built_lib.mb_settings_default(C.byref(s))
    d = PhysicsPlugin.from_c(s)
    ref = PhysicsPlugin()
    assert d.number_of_grids_one_dimension == 128 == ref.number_of_grids_one_dimension
    assert d.grid_size == 8 and d.half_map_height == 16 and d.max_number_of_agents == 16384
    assert d.enable_simulation and not d.enable_spring
    for k in ["e_envir", "e_agent", "k_agent", "c_agent", "r_agent", "time_delta"]:
        assert np.float32(getattr(d, k)) == np.float32(getattr(ref, k)), k
    assert tuple(np.float32(d.gravity)) == tuple(np.float32(ref.gravity))


def test_settings_helpers():
    s = PhysicsSettings(number_of_grids_one_dimension=1024, grid_size=1, half_map_height=8,
                        max_number_of_agents=1 << 20)
    assert s.map_size_u() == 1024 and s.half_map_size_u() == 512
    assert s.max_number_of_grids_on_dimension() == 1024
    assert s.map_height() == 16.0


QUANT_CASES = [
    PhysicsPlugin(),
    PhysicsPlugin(time_delta=1 / 60, gravity=(0.0, -9.81, 0.0), e_envir=0.8, e_agent=0.8),
    PhysicsPlugin(enable_spring=True, k_agent=1000.0, c_agent=5.0, r_agent=0.9),
    PhysicsPlugin(time_delta=1 / 15, e_envir=1.5, k_agent=400.0, c_agent=4.0, r_agent=1.0),
    PhysicsPlugin(gravity=(1.2345, -123.4567, 0.0004), e_envir=-0.5, c_agent=float("nan")),
    PhysicsPlugin(number_of_grids_one_dimension=7, grid_size=3, half_map_height=1),
    PhysicsPlugin(exact_constants=True, time_delta=1 / 60, gravity=(0.0, -9.81, 0.0)),
]


@pytest.mark.parametrize("plugin", QUANT_CASES)
def test_quantisation_matches_oracle(built_lib, plugin):
    """CompiledConsts::shader_defs (src/physics/mod.rs:459-485): x1000, truncate, /1000."""
    from bevy_millions_ball_gb300 import quantize

    ours = quantize(plugin)
    ref = oracle.quantize(plugin.to_c())
    assert bytes(ours) == bytes(ref)


def test_quantisation_reference_values(built_lib):
    from bevy_millions_ball_gb300 import quantize

    c = quantize(PhysicsPlugin(time_delta=1 / 60, gravity=(0.0, -9.81, 0.0), e_envir=0.8))
    assert c.time_delta == np.float32(0.016)  # 1/60 runs as 0.016
    assert c.gravity[1] == np.float32(-9.81)
    assert c.e_envir == np.float32(0.8)
    c = quantize(PhysicsPlugin(time_delta=1 / 120))
    assert c.time_delta == np.float32(0.008)
    c = quantize(PhysicsPlugin(number_of_grids_one_dimension=7, grid_size=3))
    assert c.half_map_size == np.float32(10.0)  # (7*3)/2 in u32


def test_pack_vfme_roundtrip():
    rng = np.random.default_rng(0)
    v = rng.standard_normal((100, 3)).astype(np.float32)
    f = rng.standard_normal((100, 3)).astype(np.float32)
    q = pack_vfme(v, f, 2.0)
    v2, f2, m2 = unpack_vfme(q)
    np.testing.assert_array_equal(v2, v.astype(np.float16).astype(np.float32))
    np.testing.assert_array_equal(f2, f.astype(np.float16).astype(np.float32))
    assert np.all(m2 == 2.0)
    assert np.all((q[:, 3] >> 16) == 0)


def test_scene_generators():
    sc = scenes.plain_uniform(4096, 64, seed=1)
    assert sc.pos_scale.shape == (4096, 4) and sc.vfme.dtype == np.uint32
    hs = 32
    assert np.all(sc.pos_scale[:, 0] < hs) and np.all(sc.pos_scale[:, 0] >= -hs)
    assert np.all(sc.pos_scale[:, 1] >= 0) and np.all(sc.pos_scale[:, 1] < 16)
    v, _, m = unpack_vfme(sc.vfme)
    assert abs(float(np.std(v)) - 0.016) < 0.002 and np.all(m == 1.0)
    cl = scenes.plain_clustered(8192, 128, seed=2)
    assert cl.plugin.enable_spring and cl.plugin.k_agent == 1000.0
    b = scenes.batch(8, seed=3)
    for s in b:
        n = s.n
        N = s.plugin.number_of_grids_one_dimension
        assert N * N >= n and N == scenes.next_pow2(math.isqrt(n - 1) + 1)
        assert s.plugin.half_map_height in (4, 8, 16)
