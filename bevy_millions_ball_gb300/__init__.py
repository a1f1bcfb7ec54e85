"""GB300-native per-step sphere-collision pipeline (bevy_millions_ball's physics passes).

Host-side mirror of the reference plugin interface:

* :class:`PhysicsPlugin` / :class:`PhysicsSettings` — the reference's
  ``PhysicsPlugin`` fields and defaults (src/physics/mod.rs:53-109) and the
  runtime ``PhysicsSettings`` helpers (mod.rs:294-400).
* :class:`World` — one scene resident on the GPU with a headless ``step()``; it
  stands in for ``PhysicsNode::run`` (mod.rs:846-912), which the reference only
  runs from its render graph.

Everything computes in ``libmillionsball.so`` (hand-written sm_103a kernels behind
the C ABI in ``include/millionsball.h``); this module only marshals arguments.
"""

from __future__ import annotations

import ctypes as C
import dataclasses
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from ._abi import MB_DEVICE, MB_HOST, MbConsts, MbError, MbServerConfig, MbServerStats, MbSettings, MbTuning

__all__ = [
    "PhysicsPlugin",
    "PhysicsSettings",
    "World",
    "SortPlan",
    "Batch",
    "Server",
    "MbError",
    "pack_vfme",
    "unpack_vfme",
    "quantize",
    "library",
    "save_png",
]


def library() -> C.CDLL:
    return _abi.load()


@dataclass
class PhysicsPlugin:
    """Fields and defaults of the reference ``PhysicsPlugin`` (src/physics/mod.rs:53-109)."""

    enable_simulation: bool = True
    enable_spring: bool = False
    number_of_grids_one_dimension: int = 128
    grid_size: int = 8
    half_map_height: int = 16
    gravity: tuple = (0.0, -9.8, 0.0)
    e_envir: float = 0.90
    e_agent: float = 0.95
    k_agent: float = 25.0
    c_agent: float = 0.1
    r_agent: float = 0.9
    max_number_of_agents: int = 16 * 1024
    time_delta: float = 1.0 / 120.0
    # not in the reference: use the f32 values as given instead of the x1000 quantisation
    exact_constants: bool = False

    def to_c(self) -> MbSettings:
        s = MbSettings()
        s.max_number_of_agents = int(self.max_number_of_agents)
        s.number_of_grids_one_dimension = int(self.number_of_grids_one_dimension)
        s.grid_size = int(self.grid_size)
        s.half_map_height = int(self.half_map_height)
        for i in range(3):
            s.gravity[i] = float(self.gravity[i])
        s.e_envir, s.e_agent = float(self.e_envir), float(self.e_agent)
        s.k_agent, s.c_agent, s.r_agent = float(self.k_agent), float(self.c_agent), float(self.r_agent)
        s.time_delta = float(self.time_delta)
        s.enable_simulation = 1 if self.enable_simulation else 0
        s.enable_spring = 1 if self.enable_spring else 0
        s.exact_constants = 1 if self.exact_constants else 0
        return s

    @classmethod
    def from_c(cls, s: MbSettings) -> "PhysicsPlugin":
        return cls(
            enable_simulation=bool(s.enable_simulation),
            enable_spring=bool(s.enable_spring),
            number_of_grids_one_dimension=s.number_of_grids_one_dimension,
            grid_size=s.grid_size,
            half_map_height=s.half_map_height,
            gravity=tuple(s.gravity),
            e_envir=s.e_envir,
            e_agent=s.e_agent,
            k_agent=s.k_agent,
            c_agent=s.c_agent,
            r_agent=s.r_agent,
            max_number_of_agents=s.max_number_of_agents,
            time_delta=s.time_delta,
            exact_constants=bool(s.exact_constants),
        )

    def replace(self, **kw) -> "PhysicsPlugin":
        return dataclasses.replace(self, **kw)


class PhysicsSettings(PhysicsPlugin):
    """Runtime settings with the reference's map helpers (src/physics/mod.rs:365-400)."""

    def max_number_of_grids_on_dimension(self) -> int:
        import math

        return math.isqrt(self.max_number_of_agents)

    def map_size_u(self) -> int:
        return self.number_of_grids_one_dimension * self.grid_size

    def half_map_size_u(self) -> int:
        return self.map_size_u() // 2

    def map_size(self) -> float:
        return float(self.map_size_u())

    def half_map_size(self) -> float:
        return float(self.half_map_size_u())

    def half_map_height_f(self) -> float:
        return float(self.half_map_height)

    def map_height(self) -> float:
        return 2.0 * float(self.half_map_height)


def save_png(path, rgba: np.ndarray) -> None:
    """Write an (H, W, 4) uint8 image as a PNG file (zlib, no other dependency)."""
    import struct
    import zlib

    h, w = rgba.shape[:2]
    raw = b"".join(b"\x00" + np.ascontiguousarray(rgba[y]).tobytes() for y in range(h))

    def chunk(tag: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
                chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))


def quantize(plugin: PhysicsPlugin) -> MbConsts:
    """Constants as the kernels use them (CompiledConsts, src/physics/mod.rs:459-485)."""
    lib = library()
    out = MbConsts()
    _abi.check(lib, lib.mb_quantize_settings(C.byref(plugin.to_c()), C.byref(out)))
    return out


def pack_vfme(velocity, force, mass) -> np.ndarray:
    """pack_vfme (src/physics/mod.rs:214-239): f16 (RNE) pairs (vx,vy) (vz,fx) (fy,fz) (m,0)."""
    v = np.asarray(velocity, np.float32).reshape(-1, 3)
    f = np.asarray(force, np.float32).reshape(-1, 3)
    m = np.broadcast_to(np.asarray(mass, np.float32), (v.shape[0],))
    h = np.zeros((v.shape[0], 8), np.float16)
    h[:, 0:3] = v.astype(np.float16)
    h[:, 3:6] = f.astype(np.float16)
    h[:, 6] = m.astype(np.float16)
    return np.ascontiguousarray(h).view(np.uint32).reshape(-1, 4).copy()


def unpack_vfme(vfme: np.ndarray):
    """Inverse of :func:`pack_vfme`: (velocity (n,3), force (n,3), mass (n,)) as float32."""
    h = np.ascontiguousarray(vfme, np.uint32).view(np.float16).reshape(-1, 8).astype(np.float32)
    return h[:, 0:3].copy(), h[:, 3:6].copy(), h[:, 6].copy()


def _stream_handle(stream) -> int:
    if stream is None:
        return 0
    if isinstance(stream, int):
        return stream
    return int(getattr(stream, "cuda_stream", stream))


class _DeviceArray:
    """A view of library-owned device memory (CUDA array interface v3).  It is
    exported writable because torch rejects read-only device arrays; a write
    changes the world's current state in place (no INIT frame follows, unlike
    set_state)."""

    def __init__(self, ptr: int, shape, typestr: str, owner):
        self._owner = owner  # keeps the world alive while the view exists
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 3, "strides": None, "stream": None}


class World:
    """One scene resident on the GPU (the reference plugin's buffers + per-frame node)."""

    def __init__(self, plugin: PhysicsPlugin, stream=None):
        self._lib = library()
        self.n = int(plugin.max_number_of_agents)
        self._h = C.c_void_p()
        _abi.check(self._lib, self._lib.mb_create(C.byref(plugin.to_c()), _stream_handle(stream), C.byref(self._h)))

    # -- lifecycle
    def close(self) -> None:
        if self._h:
            self._lib.mb_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int) -> None:
        _abi.check(self._lib, st, self._h)

    # -- settings
    @property
    def settings(self) -> PhysicsPlugin:
        s = MbSettings()
        self._check(self._lib.mb_get_settings(self._h, C.byref(s)))
        return PhysicsPlugin.from_c(s)

    def set_settings(self, plugin: PhysicsPlugin) -> None:
        self._check(self._lib.mb_set_settings(self._h, C.byref(plugin.to_c())))

    @property
    def tuning(self) -> MbTuning:
        t = MbTuning()
        self._check(self._lib.mb_get_tuning(self._h, C.byref(t)))
        return t

    def set_tuning(self, digit_bits_max: int | None = None, collide_block: int | None = None,
                   sort_algorithm: int | None = None, frames_per_launch: int | None = None,
                   state_gather: int | None = None, frame_kernel: int | None = None,
                   scatter_agents: int | None = None) -> None:
        t = self.tuning
        if scatter_agents is not None:
            t.scatter_agents = scatter_agents
        if state_gather is not None:
            t.state_gather = state_gather
        if frame_kernel is not None:
            t.frame_kernel = frame_kernel
        if digit_bits_max is not None:
            t.digit_bits_max = digit_bits_max
        if collide_block is not None:
            t.collide_block = collide_block
        if sort_algorithm is not None:
            t.sort_algorithm = sort_algorithm
        if frames_per_launch is not None:
            t.frames_per_launch = frames_per_launch
        self._check(self._lib.mb_set_tuning(self._h, C.byref(t)))

    def autotune(self, frames: int = 16) -> dict:
        """mb_autotune: time every candidate tuning on this scene, keep the state,
        apply the fastest.  Returns the chosen tuning and each candidate's ms/frame."""
        best = MbTuning()
        ms = (C.c_float * _abi.MB_TUNE_CANDIDATES)()
        tried = (MbTuning * _abi.MB_TUNE_CANDIDATES)()
        self._check(self._lib.mb_autotune(self._h, frames, C.byref(best), ms, tried))
        desc = lambda t: {"sort_algorithm": t.sort_algorithm, "digit_bits_max": t.digit_bits_max,
                          "frames_per_launch": t.frames_per_launch, "state_gather": t.state_gather,
                          "frame_kernel": t.frame_kernel, "collide_block": t.collide_block,
                          "scatter_agents": max(t.scatter_agents, 1)}
        return {"best": desc(best), "candidates": [dict(desc(t), ms_per_frame=float(m)) for t, m in zip(tried, ms)]}

    # -- state
    def set_state(self, pos_scale: np.ndarray, vfme: np.ndarray) -> None:
        p = np.ascontiguousarray(pos_scale, np.float32)
        q = np.ascontiguousarray(vfme, np.uint32)
        if p.size != 4 * self.n or q.size != 4 * self.n:
            raise ValueError(f"expected {self.n} x 4 arrays")
        self._check(self._lib.mb_set_state(self._h, p.ctypes.data, q.ctypes.data, MB_HOST))

    def set_state_device(self, pos_ptr: int, vfme_ptr: int) -> None:
        self._check(self._lib.mb_set_state(self._h, pos_ptr, vfme_ptr, MB_DEVICE))

    def get_state(self):
        p = np.empty((self.n, 4), np.float32)
        q = np.empty((self.n, 4), np.uint32)
        self._check(self._lib.mb_get_state(self._h, p.ctypes.data, q.ctypes.data, MB_HOST))
        return p, q

    def get_state_device(self, pos_ptr: int, vfme_ptr: int) -> None:
        self._check(self._lib.mb_get_state(self._h, pos_ptr, vfme_ptr, MB_DEVICE))

    def device_buffers(self):
        a, b = C.c_void_p(), C.c_void_p()
        self._check(self._lib.mb_device_buffers(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def device_state(self):
        """The current state as zero-copy device arrays (the renderer's input,
        physics_ball/mod.rs:709-740): positions+radius (n, 4) float32 and packed
        velocity/force/mass (n, 4) uint32, exposed through
        __cuda_array_interface__ (e.g. torch.as_tensor(pos, device="cuda")).
        Valid until the next step, upload or close; in the order of the last
        frame's sorted slots."""
        a, b = self.device_buffers()
        return _DeviceArray(a, (self.n, 4), "<f4", self), _DeviceArray(b, (self.n, 4), "<u4", self)

    def render_topdown(self, width: int, height: int, window=None):
        """mb_render_topdown: a width x height RGBA8 image (H, W, 4) uint8 and the
        surface height map (H, W) float32 of the current state, seen straight down
        onto the x/z window (x0, z0, x1, z1) (default: the whole map)."""
        if window is None:
            s = self.settings
            hs = s.number_of_grids_one_dimension * s.grid_size / 2.0
            window = (-hs, -hs, hs, hs)
        x0, z0, x1, z1 = (float(v) for v in window)
        img = np.empty((height, width), np.uint32)
        hmap = np.empty((height, width), np.float32)
        self._check(self._lib.mb_render_topdown(self._h, width, height, x0, z0, x1, z1, img.ctypes.data,
                                                hmap.ctypes.data, MB_HOST))
        return img.view(np.uint8).reshape(height, width, 4), hmap

    def render_view(self, width: int, height: int, eye=None, target=None, fov_y_degrees: float = 0.0):
        """mb_render_view: a width x height RGBA8 image (H, W, 4) uint8 and the depth
        (distance along each pixel's ray, 0 for the clear colour) (H, W) float32 of
        the current state through a perspective camera; by default the reference
        view (eye (0, 64, 64) looking at the origin, 45-degree field of view)."""
        img = np.empty((height, width), np.uint32)
        depth = np.empty((height, width), np.float32)
        e = None if eye is None else np.ascontiguousarray(eye, np.float32)
        t = None if target is None else np.ascontiguousarray(target, np.float32)
        self._check(self._lib.mb_render_view(self._h, width, height, None if e is None else e.ctypes.data,
                                             None if t is None else t.ctypes.data, float(fov_y_degrees),
                                             img.ctypes.data, depth.ctypes.data, MB_HOST))
        return img.view(np.uint8).reshape(height, width, 4), depth

    # -- stepping
    def step(self, k: int = 1) -> None:
        self._check(self._lib.mb_step(self._h, int(k)))

    def sync(self) -> None:
        self._check(self._lib.mb_sync(self._h))

    @property
    def time(self) -> int:
        return int(self._lib.mb_time(self._h))

    def set_profiling(self, on: bool = True) -> None:
        self._check(self._lib.mb_set_profiling(self._h, 1 if on else 0))

    def last_frame_times(self):
        """(sort_ms, cells_ms, physics_ms) of the most recent frame (profiling on)."""
        ms = (C.c_float * 3)()
        self._check(self._lib.mb_last_frame_times(self._h, ms))
        return tuple(ms)

    @property
    def kernels_per_frame(self) -> int:
        return int(self._lib.mb_kernels_per_frame(self._h))

    def debug(self, cells: int | None = None):
        s = self.settings
        cells = cells or s.number_of_grids_one_dimension ** 2
        keys = np.empty(self.n, np.uint32)
        perm = np.empty(self.n, np.uint32)
        start = np.empty(cells, np.uint32)
        close = np.empty(cells, np.uint32)
        self._check(self._lib.mb_get_debug(self._h, keys.ctypes.data, perm.ctypes.data, start.ctypes.data,
                                           close.ctypes.data, MB_HOST))
        return {"keys": keys, "perm": perm, "start": start, "close": close}


class SortPlan:
    """Stage API: stable sort + cell-range build on device buffers (mb_sort_and_hash)."""

    def __init__(self, max_keys: int, max_cells: int):
        self._lib = library()
        self._h = C.c_void_p()
        _abi.check(self._lib, self._lib.mb_sort_plan_create(int(max_keys), int(max_cells), C.byref(self._h)))

    def run(self, keys_ptr: int, vals_ptr: int | None, n: int, cells: int, sorted_keys_ptr: int,
            sorted_vals_ptr: int, start_ptr: int | None, close_ptr: int | None, stream=None) -> None:
        _abi.check(self._lib, self._lib.mb_sort_and_hash(self._h, keys_ptr, vals_ptr, int(n), int(cells),
                                                         sorted_keys_ptr, sorted_vals_ptr, start_ptr,
                                                         close_ptr, _stream_handle(stream)))

    def status(self, stream=None) -> None:
        """mb_sort_plan_status: raises MbError (MB_ERR_TIMEOUT) if a bounded device
        wait of the plan's sorts gave up since the last check (and clears it)."""
        _abi.check(self._lib, self._lib.mb_sort_plan_status(self._h, _stream_handle(stream)))

    def assemble_segments(self, sorted_keys_ptr: int, n: int, segs_ptr: int, key_seg_map_ptr: int,
                          num_segs_ptr: int, stream=None) -> None:
        """mb_assemble_segments: one segment per run of equal sorted keys (device pointers)."""
        _abi.check(self._lib, self._lib.mb_assemble_segments(self._h, sorted_keys_ptr, int(n), segs_ptr,
                                                             key_seg_map_ptr, num_segs_ptr, _stream_handle(stream)))

    def close(self) -> None:
        if self._h:
            self._lib.mb_sort_plan_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many independent scenes stepped together (mb_batch_*); each evolves exactly as alone."""

    def __init__(self, plugins, capacity_agents: int = 0, capacity_cells: int = 0, capacity_scenes: int = 0,
                 stream=None):
        self._lib = library()
        arr = (MbSettings * max(len(plugins), 1))(*[p.to_c() for p in plugins])
        self._h = C.c_void_p()
        self.sizes = [int(p.max_number_of_agents) for p in plugins]
        self.cells = [int(p.number_of_grids_one_dimension) ** 2 for p in plugins]
        _abi.check(self._lib, self._lib.mb_batch_create(arr, len(plugins), capacity_agents, capacity_cells,
                                                        capacity_scenes, _stream_handle(stream), C.byref(self._h)))

    def _check(self, st):
        _abi.check(self._lib, st)

    def add_scene(self, plugin: PhysicsPlugin) -> int:
        idx = C.c_uint32()
        self._check(self._lib.mb_batch_add_scene(self._h, C.byref(plugin.to_c()), C.byref(idx)))
        self.sizes.append(int(plugin.max_number_of_agents))
        self.cells.append(int(plugin.number_of_grids_one_dimension) ** 2)
        return idx.value

    def set_state(self, scene: int, pos_scale: np.ndarray, vfme: np.ndarray) -> None:
        p = np.ascontiguousarray(pos_scale, np.float32)
        q = np.ascontiguousarray(vfme, np.uint32)
        self._check(self._lib.mb_batch_set_state(self._h, scene, p.ctypes.data, q.ctypes.data, MB_HOST))

    def get_state(self, scene: int):
        n = self.sizes[scene]
        p = np.empty((n, 4), np.float32)
        q = np.empty((n, 4), np.uint32)
        self._check(self._lib.mb_batch_get_state(self._h, scene, p.ctypes.data, q.ctypes.data, MB_HOST))
        return p, q

    def set_active(self, scene: int, active: bool) -> None:
        self._check(self._lib.mb_batch_set_active(self._h, scene, 1 if active else 0))

    def step(self, k: int = 1) -> None:
        self._check(self._lib.mb_batch_step(self._h, int(k)))

    def sync(self) -> None:
        self._check(self._lib.mb_batch_sync(self._h))

    def time(self, scene: int) -> int:
        return int(self._lib.mb_batch_time(self._h, scene))

    def debug(self, scene: int):
        n, c = self.sizes[scene], self.cells[scene]
        keys, perm = np.empty(n, np.uint32), np.empty(n, np.uint32)
        start, close = np.empty(c, np.uint32), np.empty(c, np.uint32)
        self._check(self._lib.mb_batch_get_debug(self._h, scene, keys.ctypes.data, perm.ctypes.data,
                                                 start.ctypes.data, close.ctypes.data, MB_HOST))
        return {"keys": keys, "perm": perm, "start": start, "close": close}

    def memory(self) -> int:
        b = C.c_uint64()
        self._check(self._lib.mb_batch_memory(self._h, C.byref(b)))
        return b.value

    @property
    def tuning(self) -> MbTuning:
        t = MbTuning()
        self._check(self._lib.mb_batch_get_tuning(self._h, C.byref(t)))
        return t

    def set_tuning(self, frames_per_launch: int | None = None, collide_block: int | None = None,
                   scatter_agents: int | None = None, sort_algorithm: int | None = None) -> None:
        t = self.tuning
        if sort_algorithm is not None:
            t.sort_algorithm = sort_algorithm
        if scatter_agents is not None:
            t.scatter_agents = scatter_agents
        if frames_per_launch is not None:
            t.frames_per_launch = frames_per_launch
        if collide_block is not None:
            t.collide_block = collide_block
        self._check(self._lib.mb_batch_set_tuning(self._h, C.byref(t)))

    def autotune(self, frames: int = 16) -> dict:
        """mb_batch_autotune: time frames_per_launch x collide_block (and scatter_agents)
        on the pool's own scenes (states restored), apply the fastest; returns it and
        every candidate's ms/frame."""
        n = _abi.MB_BATCH_TUNE_CANDIDATES
        best, ms, tried = MbTuning(), (C.c_float * n)(), (MbTuning * n)()
        self._check(self._lib.mb_batch_autotune(self._h, frames, C.byref(best), ms, tried))
        desc = lambda t: {"sort_algorithm": t.sort_algorithm, "frames_per_launch": t.frames_per_launch,
                          "collide_block": t.collide_block, "scatter_agents": max(t.scatter_agents, 1)}
        return {"best": desc(best), "candidates": [dict(desc(t), ms_per_frame=float(m)) for t, m in zip(tried, ms)]}

    def close(self) -> None:
        if self._h:
            self._lib.mb_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Request-serving loop over one batch pool (mb_server_*)."""

    def __init__(self, budget_bytes: int, max_scenes: int = 4096, max_agents: int = 0, max_cells: int = 0,
                 stream=None):
        self._lib = library()
        cfg = MbServerConfig(budget_bytes=int(budget_bytes), max_scenes=max_scenes, max_agents=max_agents,
                             max_cells=max_cells)
        self._h = C.c_void_p()
        self.sizes = {}
        _abi.check(self._lib, self._lib.mb_server_create(C.byref(cfg), _stream_handle(stream), C.byref(self._h)))

    def create(self, plugin: PhysicsPlugin, pos_scale: np.ndarray, vfme: np.ndarray):
        """Submit a create-scene request: returns (scene handle, request id)."""
        p = np.ascontiguousarray(pos_scale, np.float32)
        q = np.ascontiguousarray(vfme, np.uint32)
        sc, rq = C.c_uint32(), C.c_uint64()
        _abi.check(self._lib, self._lib.mb_server_submit_create(self._h, C.byref(plugin.to_c()), p.ctypes.data,
                                                                q.ctypes.data, C.byref(sc), C.byref(rq)))
        self.sizes[sc.value] = int(plugin.max_number_of_agents)
        return sc.value, rq.value

    def advance(self, scene: int, k: int) -> int:
        rq = C.c_uint64()
        _abi.check(self._lib, self._lib.mb_server_submit_advance(self._h, scene, int(k), C.byref(rq)))
        return rq.value

    def wait(self, request: int, timeout: float = 600.0) -> float:
        """Block until the request is done; returns its latency in seconds."""
        lat = C.c_double()
        _abi.check(self._lib, self._lib.mb_server_wait(self._h, request, timeout, C.byref(lat)))
        return lat.value

    def get_state(self, scene: int):
        n = self.sizes[scene]
        p = np.empty((n, 4), np.float32)
        q = np.empty((n, 4), np.uint32)
        _abi.check(self._lib, self._lib.mb_server_get_state(self._h, scene, p.ctypes.data, q.ctypes.data))
        return p, q

    def stats(self) -> MbServerStats:
        st = MbServerStats()
        _abi.check(self._lib, self._lib.mb_server_get_stats(self._h, C.byref(st)))
        return st

    def close(self) -> None:
        if self._h:
            self._lib.mb_server_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
