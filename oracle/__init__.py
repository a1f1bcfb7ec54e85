"""CPU oracle — TEST INFRASTRUCTURE ONLY.

A C++ restatement of the reference's per-frame passes (see oracle.h for what it
follows, line by line).  Only tests/, ``__graft_entry__.smoke()`` and bench.py's
CPU-baseline leg may use it, always as the checker or the timed CPU reference,
never as the product.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from bevy_millions_ball_gb300._abi import MbConsts, MbSettings

from .build_oracle import LIB as LIB_PATH
from .build_oracle import build

vp, u32, i64 = C.c_void_p, C.c_uint32, C.c_int64

_SIG = {
    "mbo_quantize": (C.c_int, [C.POINTER(MbSettings), C.POINTER(MbConsts)]),
    "mbo_f32_to_f16": (C.c_uint16, [C.c_float]),
    "mbo_f16_to_f32": (C.c_float, [C.c_uint16]),
    "mbo_cell_key": (u32, [C.POINTER(MbConsts), C.c_float, C.c_float]),
    "mbo_hash3f1u": (None, [u32, C.POINTER(C.c_float)]),
    "mbo_radix_sort": (None, [vp, vp, u32, u32, vp, vp, C.c_int]),
    "mbo_spatial_hash": (None, [vp, u32, u32, vp, vp]),
    "mbo_physics": (None, [C.POINTER(MbConsts), C.c_int, u32, vp, vp, vp, vp, vp, vp, vp, vp, C.c_int]),
    "mbo_create": (vp, [C.POINTER(MbSettings)]),
    "mbo_destroy": (None, [vp]),
    "mbo_set_settings": (C.c_int, [vp, C.POINTER(MbSettings)]),
    "mbo_set_state": (C.c_int, [vp, vp, vp]),
    "mbo_get_state": (C.c_int, [vp, vp, vp]),
    "mbo_step": (C.c_int, [vp, u32, C.c_int]),
    "mbo_get_debug": (C.c_int, [vp, vp, vp, vp, vp]),
    "mbo_time": (i64, [vp]),
    "mbo_hardware_threads": (C.c_int, []),
    "mbo_render_topdown": (None, [vp, u32, u32, u32, C.c_float, C.c_float, C.c_float, C.c_float, vp, vp, vp]),
    "mbo_reference_view": (None, [vp, vp, vp, vp]),
    "mbo_render_view": (None, [vp, u32, u32, u32, vp, vp, C.c_float, vp, C.c_float, C.c_float, vp, vp, vp]),
}

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = build()
        L = C.CDLL(str(path))
        for name, (res, args) in _SIG.items():
            fn = getattr(L, name)
            fn.restype, fn.argtypes = res, args
        _lib = L
    return _lib


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


def quantize(settings: MbSettings) -> MbConsts:
    c = MbConsts()
    lib().mbo_quantize(C.byref(settings), C.byref(c))
    return c


def radix_sort(keys: np.ndarray, vals: np.ndarray | None = None, passes: int = 3, threads: int = 0):
    keys = np.ascontiguousarray(keys, np.uint32)
    n = keys.size
    ko, vo = np.empty(n, np.uint32), np.empty(n, np.uint32)
    vv = None if vals is None else np.ascontiguousarray(vals, np.uint32)
    lib().mbo_radix_sort(_p(keys), None if vv is None else _p(vv), n, passes, _p(ko), _p(vo), threads)
    return ko, vo


def spatial_hash(sorted_keys: np.ndarray, cells: int):
    sk = np.ascontiguousarray(sorted_keys, np.uint32)
    start, close = np.empty(cells, np.uint32), np.empty(cells, np.uint32)
    lib().mbo_spatial_hash(_p(sk), sk.size, cells, _p(start), _p(close))
    return start, close


class OracleWorld:
    """CPU world with the reference's frame semantics (sort -> hash -> INIT/LOOP physics)."""

    def __init__(self, settings: MbSettings, threads: int = 0):
        self._lib = lib()
        self._h = self._lib.mbo_create(C.byref(settings))
        if not self._h:
            raise ValueError("oracle rejected the settings")
        self.n = settings.max_number_of_agents
        self.cells = settings.number_of_grids_one_dimension ** 2
        self.threads = threads

    def set_settings(self, settings: MbSettings) -> None:
        if self._lib.mbo_set_settings(self._h, C.byref(settings)):
            raise ValueError("oracle rejected the settings")
        self.cells = settings.number_of_grids_one_dimension ** 2

    def set_state(self, pos: np.ndarray, vfme: np.ndarray) -> None:
        p = np.ascontiguousarray(pos, np.float32)
        q = np.ascontiguousarray(vfme, np.uint32)
        self._lib.mbo_set_state(self._h, _p(p), _p(q))

    def step(self, k: int = 1) -> None:
        if self._lib.mbo_step(self._h, k, self.threads):
            raise RuntimeError("oracle step without state")

    def get_state(self):
        p = np.empty((self.n, 4), np.float32)
        q = np.empty((self.n, 4), np.uint32)
        self._lib.mbo_get_state(self._h, _p(p), _p(q))
        return p, q

    def debug(self):
        keys, perm = np.empty(self.n, np.uint32), np.empty(self.n, np.uint32)
        start, close = np.empty(self.cells, np.uint32), np.empty(self.cells, np.uint32)
        self._lib.mbo_get_debug(self._h, _p(keys), _p(perm), _p(start), _p(close))
        return {"keys": keys, "perm": perm, "start": start, "close": close}

    @property
    def time(self) -> int:
        return int(self._lib.mbo_time(self._h))

    def close(self) -> None:
        if self._h:
            self._lib.mbo_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def render_topdown(pos: np.ndarray, width: int, height: int, x0: float, z0: float, x1: float, z1: float):
    """Top-down impostor render: (rgba u32 (h, w), height f32 (h, w), winner u32 (h, w): sphere index + 1)."""
    p = np.ascontiguousarray(pos, np.float32)
    rgba = np.empty((height, width), np.uint32)
    hmap = np.empty((height, width), np.float32)
    win = np.empty((height, width), np.uint32)
    lib().mbo_render_topdown(_p(p), p.shape[0], width, height, x0, z0, x1, z1, _p(rgba), _p(hmap), _p(win))
    return rgba, hmap, win


def reference_view():
    """The reference's camera and light: (eye (3,), target (3,), fov degrees, unit vector towards the light (3,))."""
    eye, target, light = (np.empty(3, np.float32) for _ in range(3))
    fov = np.empty(1, np.float32)
    lib().mbo_reference_view(_p(eye), _p(target), _p(fov), _p(light))
    return eye, target, float(fov[0]), light


def render_view(pos: np.ndarray, width: int, height: int, half_map_size: float, map_top: float, eye=None,
                target=None, fov_degrees: float = 0.0):
    """Perspective impostor render: (rgba u32 (h, w), depth f32 (h, w), winner u32 (h, w): sphere index + 1)."""
    e0, t0, f0, light = reference_view()
    eye = e0 if eye is None else np.ascontiguousarray(eye, np.float32)
    target = t0 if target is None else np.ascontiguousarray(target, np.float32)
    fov = f0 if fov_degrees <= 0 else float(fov_degrees)
    p = np.ascontiguousarray(pos, np.float32)
    rgba = np.empty((height, width), np.uint32)
    depth = np.empty((height, width), np.float32)
    win = np.empty((height, width), np.uint32)
    lib().mbo_render_view(_p(p), p.shape[0], width, height, _p(eye), _p(target), fov, _p(light), half_map_size,
                          map_top, _p(rgba), _p(depth), _p(win))
    return rgba, depth, win


def hardware_threads() -> int:
    return int(lib().mbo_hardware_threads())
